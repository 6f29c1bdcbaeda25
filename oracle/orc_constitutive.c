/*
 * CPU oracle (test infrastructure only): restatement of the reference's
 * per-integration-point Mohr-Coulomb update.
 *
 * The arithmetic follows the reference headers operation by operation
 * (same association, same constants, same branch tests) so that the result
 * is bit-identical to the reference CPU build; the CUDA product reproduces
 * the same sequence in a plane-strain-reduced form.  Deviations from the
 * reference, each one giving undefined behaviour a defined meaning:
 *   - gamma[2] of the edge return mappings starts at 0
 *     (FunctionsSigmaProjection.h:103, 205 leave it uninitialised);
 *   - alpha / m_hardening accumulates from 0
 *     (TPZConstitutiveLawProcessor.cpp:160 leaves it uninitialised);
 *   - abs() on the cubic residual is the floating-point absolute value
 *     (FunctionsSpectralDecomp.h:80,89 would bind integer abs without
 *     `using std::abs`).
 * Compile with -ffp-contract=off.
 */
#include <math.h>
#include <string.h>
#include "ipfem_oracle.h"

enum { XX = 0, XY = 1, XZ = 2, YY = 3, YZ = 4, ZZ = 5 };

void orc_mc_from_angles(double cohesion, double phi, double psi, orc_mc *out)
{
    out->cohesion = cohesion;
    out->sinphi = sin(phi);
    out->cosphi = cos(phi);
    out->tanphi = tan(phi);
    out->sinpsi = sin(psi);
}

void orc_lame_from_engineering(double E, double nu, orc_elastic *out)
{
    out->lambda = (E * nu) / ((1.0 + nu) * (1.0 - 2.0 * nu));
    out->mu = E / (2.0 * (1.0 + nu));
}

/* ------------------------------------------------ FunctionsStressStrain.h */

/* ComposeStrain, FunctionsStressStrain.h:10-24 (dim == 2 branch) */
static void compose_strain(const double *d, double *full)
{
    full[XX] = d[0];
    full[XY] = d[1];
    full[XZ] = 0;
    full[YY] = d[2];
    full[YZ] = 0;
    full[ZZ] = 0;
}

/* ElasticStrain, FunctionsStressStrain.h:29-33 */
static void elastic_strain(const double *pl, const double *eps, double *el)
{
    for (int i = 0; i < 6; i++) el[i] = eps[i] - pl[i];
}

/* PlasticStrain, FunctionsStressStrain.h:38-42 */
static void plastic_strain(const double *eps, const double *el, double *pl)
{
    for (int i = 0; i < 6; i++) pl[i] = eps[i] - el[i];
}

/* ComputeTrialStress, FunctionsStressStrain.h:47-55 */
static void trial_stress(const double *e, double *s, double mu, double lambda)
{
    s[XX] = (lambda + 2 * mu) * e[XX] + lambda * e[YY] + lambda * e[ZZ];
    s[YY] = lambda * e[XX] + (lambda + 2 * mu) * e[YY] + lambda * e[ZZ];
    s[ZZ] = lambda * e[XX] + lambda * e[YY] + (lambda + 2 * mu) * e[ZZ];
    s[XY] = mu * e[XY];
    s[XZ] = mu * e[XZ];
    s[YZ] = mu * e[YZ];
}

/* ReconstructStressTensor, FunctionsStressStrain.h:60-68 */
static void reconstruct(const double *p, const double *v, double *s)
{
    s[XX] = (p[0] * v[0] * v[0] + p[1] * v[3] * v[3] + p[2] * v[6] * v[6]);
    s[YY] = (p[0] * v[1] * v[1] + p[1] * v[4] * v[4] + p[2] * v[7] * v[7]);
    s[ZZ] = (p[0] * v[2] * v[2] + p[1] * v[5] * v[5] + p[2] * v[8] * v[8]);
    s[XY] = (p[0] * v[0] * v[1] + p[1] * v[3] * v[4] + p[2] * v[6] * v[7]);
    s[XZ] = (p[0] * v[0] * v[2] + p[1] * v[3] * v[5] + p[2] * v[6] * v[8]);
    s[YZ] = (p[0] * v[1] * v[2] + p[1] * v[4] * v[5] + p[2] * v[7] * v[8]);
}

/* ComputeStrain (inverse elasticity), FunctionsStressStrain.h:73-81 */
static void strain_from_stress(const double *s, double *e, double mu, double lambda)
{
    e[XX] = (lambda + mu) / (3 * lambda * mu + 2 * mu * mu) * s[XX]
          - lambda / (6 * lambda * mu + 4 * mu * mu) * (s[YY] + s[ZZ]);
    e[YY] = (lambda + mu) / (3 * lambda * mu + 2 * mu * mu) * s[YY]
          - lambda / (6 * lambda * mu + 4 * mu * mu) * (s[XX] + s[ZZ]);
    e[ZZ] = (lambda + mu) / (3 * lambda * mu + 2 * mu * mu) * s[ZZ]
          - lambda / (6 * lambda * mu + 4 * mu * mu) * (s[YY] + s[XX]);
    e[XY] = 1 / mu * s[XY];
    e[XZ] = 1 / mu * s[XZ];
    e[YZ] = 1 / mu * s[YZ];
}

/* TranslateDep, FunctionsStressStrain.h:103-119 */
static void translate_dep(const double *full, double *dep)
{
    static const int ind[3] = {XX, XY, YY};
    for (int i = 0; i < 3; ++i) {
        dep[3 * i + 0] = full[XX + 6 * ind[i]];
        dep[3 * i + 1] = full[XY + 6 * ind[i]];
        dep[3 * i + 2] = full[YY + 6 * ind[i]];
    }
    dep[1] /= 2;
    dep[4] /= 2;
    dep[7] /= 2;
}

/* ---------------------------------------------- FunctionsSpectralDecomp.h */

/* Normalize, FunctionsSpectralDecomp.h:7-20 */
static void sd_normalize(double *s, double *maxel)
{
    double m = s[0];
    for (int i = 1; i < 6; i++)
        if (fabs(s[i]) > fabs(m)) m = s[i];
    if (m != 0)
        for (int i = 0; i < 6; i++) s[i] /= m;
    *maxel = m;
}

/* Interval (Gershgorin bounds), FunctionsSpectralDecomp.h:25-56 */
static void sd_interval(const double *s, double *iv)
{
    double lo[3], up[3];
    double r1 = s[XY] + s[XZ];
    lo[0] = s[XX] - fabs(r1);
    up[0] = s[XX] + fabs(r1);
    double r2 = s[XY] + s[YZ];
    lo[1] = s[YY] - fabs(r2);
    up[1] = s[YY] + fabs(r2);
    double r3 = s[XY] + s[YZ];          /* as in the reference (row 3 reuses XY) */
    lo[2] = s[ZZ] - fabs(r3);
    up[2] = s[ZZ] + fabs(r3);
    iv[0] = up[0];
    iv[1] = lo[0];
    for (int i = 1; i < 3; i++) {
        if (up[i] > iv[0]) iv[0] = up[i];
        if (lo[i] < iv[1]) iv[1] = lo[i];
    }
}

static double sd_cubic(const double *s, double x, double sxy2, double sxz2, double syz2)
{
    return -x * x * x - sxz2 * s[YY] - sxy2 * s[ZZ] - syz2 * s[XX] + 2 * s[XY] * s[XZ] * s[YZ]
           + s[XX] * s[YY] * s[ZZ] + x * x * (s[XX] + s[YY] + s[ZZ])
           + x * (sxy2 + sxz2 + syz2 - s[XX] * s[YY] - s[XX] * s[ZZ] - s[YY] * s[ZZ]);
}

/* NewtonIterations on the characteristic cubic, FunctionsSpectralDecomp.h:61-111 */
static void sd_newton(const double *iv, const double *s, double *ev, double maxel)
{
    const int numiterations = 20;
    const double tol = 10e-12;
    for (int i = 0; i < 2; i++) {
        double x = iv[i];
        int it = 0;
        double sxy2 = s[XY] * s[XY];
        double sxz2 = s[XZ] * s[XZ];
        double syz2 = s[YZ] * s[YZ];
        double f = sd_cubic(s, x, sxy2, sxz2, syz2);
        double res = fabs(f);
        while (it < numiterations && res > tol) {
            double df = -3 * x * x + sxy2 + sxz2 + syz2 - s[XX] * s[YY] - s[XX] * s[ZZ] - s[YY] * s[ZZ]
                        + 2 * x * (s[XX] + s[YY] + s[ZZ]);
            x -= f / df;
            f = sd_cubic(s, x, sxy2, sxz2, syz2);
            res = fabs(f);
            it++;
        }
        ev[i] = x;
    }
    ev[2] = s[XX] + s[YY] + s[ZZ] - ev[0] - ev[1];
    ev[0] *= maxel;
    ev[1] *= maxel;
    ev[2] *= maxel;
    for (int i = 0; i < 3; ++i)
        for (int j = i + 1; j < 3; ++j)
            if (ev[i] < ev[j]) {
                double a = ev[i];
                ev[i] = ev[j];
                ev[j] = a;
            }
}

/* Multiplicity1, FunctionsSpectralDecomp.h:116-150 */
static void sd_mult1(const double *s, double lam, double *vec)
{
    double det[3];
    det[0] = (s[XX] - lam) * (s[YY] - lam) - s[XY] * s[XY];
    det[1] = (s[XX] - lam) * (s[ZZ] - lam) - s[XZ] * s[XZ];
    det[2] = (s[YY] - lam) * (s[ZZ] - lam) - s[YZ] * s[YZ];
    double maxdet = fabs(det[0]);
    for (int i = 1; i < 3; i++)
        if (fabs(det[i]) > fabs(maxdet)) maxdet = fabs(det[i]);
    double v[3];
    if (maxdet == fabs(det[0])) {
        v[0] = 1 / det[0] * (-(s[YY] - lam) * s[XZ] + s[XY] * s[YZ]);
        v[1] = 1 / det[0] * (-(s[XX] - lam) * s[YZ] + s[XY] * s[XZ]);
        v[2] = 1;
    } else if (maxdet == fabs(det[1])) {
        v[0] = 1 / det[1] * (-(s[ZZ] - lam) * s[XY] + s[XZ] * s[YZ]);
        v[1] = 1;
        v[2] = 1 / det[1] * (-(s[XX] - lam) * s[YZ] + s[XY] * s[XZ]);
    } else {
        v[0] = 1;
        v[1] = 1 / det[2] * (-(s[ZZ] - lam) * s[XY] + s[XZ] * s[YZ]);
        v[2] = 1 / det[2] * (-(s[YY] - lam) * s[XZ] + s[XY] * s[YZ]);
    }
    double norm = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    vec[0] = v[0] / norm;
    vec[1] = v[1] / norm;
    vec[2] = v[2] / norm;
}

/* Multiplicity2, FunctionsSpectralDecomp.h:155-212.  The second norm keeps
 * the reference's v2[1]*v1[1] term (…h:203). */
static void sd_mult2(const double *s, double lam, double *vec1, double *vec2)
{
    double x[3];
    x[0] = s[XX] - lam;
    x[1] = s[YY] - lam;
    x[2] = s[ZZ] - lam;
    double maxx = fabs(x[0]);
    for (int i = 1; i < 3; i++)
        if (fabs(x[i]) > fabs(maxx)) maxx = fabs(x[i]);
    double v1[3], v2[3];
    if (maxx == fabs(x[0])) {
        v1[0] = -s[XY] / x[0]; v1[1] = 1; v1[2] = 0;
        v2[0] = -s[XZ] / x[0]; v2[1] = 0; v2[2] = 1;
    } else if (maxx == fabs(x[1])) {
        v1[0] = 1; v1[1] = -s[XY] / x[1]; v1[2] = 0;
        v2[0] = 0; v2[1] = -s[YZ] / x[1]; v2[2] = 1;
    } else {
        v1[0] = 1; v1[1] = 0; v1[2] = -s[XZ] / x[2];
        v2[0] = 0; v2[1] = 1; v2[2] = -s[YZ] / x[2];
    }
    double n1 = sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
    double n2 = sqrt(v2[0] * v2[0] + v2[1] * v1[1] + v2[2] * v2[2]);
    vec1[0] = v1[0] / n1; vec1[1] = v1[1] / n1; vec1[2] = v1[2] / n1;
    vec2[0] = v2[0] / n2; vec2[1] = v2[1] / n2; vec2[2] = v2[2] / n2;
}

/* Eigenvectors, FunctionsSpectralDecomp.h:217-256 (denormalises s in place) */
static void sd_eigenvectors(double *s, const double *ev, double *vec, double maxel)
{
    for (int i = 0; i < 6; i++) s[i] *= maxel;      /* order XX,YY,ZZ,XY,XZ,YZ is immaterial */
    if ((ev[0] == ev[1]) && (ev[1] == ev[2])) {
        memset(vec, 0, 9 * sizeof(double));
        vec[0] = 1.; vec[4] = 1.; vec[8] = 1.;
    } else {
        if (ev[0] != ev[1] && ev[0] != ev[2]) {
            sd_mult1(s, ev[0], &vec[0]);
        } else if (ev[0] == ev[1]) {
            sd_mult2(s, ev[0], &vec[0], &vec[3]);
        } else if (ev[0] == ev[2]) {
            sd_mult2(s, ev[0], &vec[0], &vec[6]);
        }
        if (ev[1] != ev[0] && ev[1] != ev[2]) {
            sd_mult1(s, ev[1], &vec[3]);
        } else if (ev[1] == ev[2]) {
            sd_mult2(s, ev[1], &vec[3], &vec[6]);
        }
        if (ev[2] != ev[0] && ev[2] != ev[1]) {
            sd_mult1(s, ev[2], &vec[6]);
        }
    }
}

/* Decomposition variant for studies (the default, 0, is the reference's
 * SpectralDecomposition, which every parity test pins).  1: for a tensor with
 * XZ = YZ = 0, which every plane-strain state is, ZZ with (0, 0, 1) and the
 * closed-form eigen-pairs of the in-plane 2x2 block, so the vectors are
 * orthonormal at any eigenvalue gap.  The reference's Newton iteration on the
 * cubic leaves roots near a double root about 3e-6 (relative) off, and its
 * Multiplicity1 then computes the two eigenvectors of a nearly repeated pair
 * one at a time from a nearly singular system: they can coincide, and the
 * reconstructed stress is then wrong by the size of the stress. */
static int g_spectral_mode = 0;
void orc_set_spectral_mode(int mode) { g_spectral_mode = mode; }

static void spectral_plane(const double *s, double *ev, double *vec)
{
    const double d = 0.5 * (s[XX] - s[YY]), m = 0.5 * (s[XX] + s[YY]);
    const double r = sqrt(d * d + s[XY] * s[XY]);
    double c = 1.0, sn = 0.0;           /* unit eigenvector of m + r */
    if (r > 0.0) {
        /* (A - (m + r) I) x = 0 for x = (d + r, b) and for x = (b, r - d):
         * take the one whose first or second entry is at least r */
        const double x = d >= 0.0 ? d + r : s[XY];
        const double y = d >= 0.0 ? s[XY] : r - d;
        const double n = sqrt(x * x + y * y);
        c = x / n;
        sn = y / n;
    }
    const double lam[3] = {m + r, m - r, s[ZZ]};
    const double v[3][3] = {{c, sn, 0.0}, {-sn, c, 0.0}, {0.0, 0.0, 1.0}};
    /* descending; m + r >= m - r, and ZZ goes after an equal in-plane value */
    int o[3] = {0, 1, 2};
    if (lam[2] > lam[0]) {
        o[0] = 2; o[1] = 0; o[2] = 1;
    } else if (lam[2] > lam[1]) {
        o[1] = 2; o[2] = 1;
    }
    for (int k = 0; k < 3; k++) {
        ev[k] = lam[o[k]];
        for (int q = 0; q < 3; q++) vec[3 * k + q] = v[o[k]][q];
    }
}

/* SpectralDecomposition, FunctionsSpectralDecomp.h:261-268 */
static void spectral(double *s, double *ev, double *vec)
{
    if (g_spectral_mode == 1 && s[XZ] == 0.0 && s[YZ] == 0.0) {
        spectral_plane(s, ev, vec);
        return;
    }
    double maxel, iv[2];
    sd_normalize(s, &maxel);
    sd_interval(s, iv);
    sd_newton(iv, s, ev, maxel);
    sd_eigenvectors(s, ev, vec, maxel);
}

/* -------------------------------------------- FunctionsSigmaProjection.h */

/* PhiPlane, FunctionsSigmaProjection.h:6-20 */
static int phi_plane(const double *ev, double *sp, const orc_mc *m)
{
    double phi = ev[0] - ev[2] + (ev[0] + ev[2]) * m->sinphi - 2. * m->cohesion * m->cosphi;
    sp[0] = ev[0];
    sp[1] = ev[1];
    sp[2] = ev[2];
    return (fabs(phi) < 1.e-12) || (phi < 0.0);
}

/* ReturnMappingMainPlane, FunctionsSigmaProjection.h:25-63 */
static int rm_main_plane(const double *st, double *sp, double *hard, const orc_mc *m,
                         double K, double G)
{
    double ev[3] = {st[0], st[1], st[2]};
    const double sinphi = m->sinphi, sinpsi = m->sinpsi, cosphi = m->cosphi;
    const double sinphi2 = sinphi * sinphi;
    const double cosphi2 = 1. - sinphi2;
    const double constA = 4. * G * (1. + sinphi * sinpsi / 3.) + 4. * K * sinphi * sinpsi;
    double phi = ev[0] - ev[2] + (ev[0] + ev[2]) * sinphi - 2. * m->cohesion * cosphi;
    double gamma = 0;
    for (int i = 0; i < 30; i++) {
        double jac = -constA - 4. * cosphi2 * 0;   /* H = 0 */
        double dgamma = -phi / jac;
        gamma += dgamma;
        phi = ev[0] - ev[2] + (ev[0] + ev[2]) * sinphi - 2. * m->cohesion * cosphi - constA * gamma;
        if (fabs(phi) < 1.e-12) break;
    }
    ev[0] -= (2. * G * (1 + sinpsi / 3.) + 2. * K * sinpsi) * gamma;
    ev[1] += (4. * G / 3. - K * 2.) * sinpsi * gamma;
    ev[2] += (2. * G * (1 - sinpsi / 3.) - 2. * K * sinpsi) * gamma;
    sp[0] = ev[0];
    sp[1] = ev[1];
    sp[2] = ev[2];
    *hard += gamma * 2. * cosphi;
    return (ev[0] > ev[1] || fabs(ev[0] - ev[1]) < 1.e-12) && (ev[1] > ev[2] || fabs(ev[1] - ev[2]) < 1.e-12);
}

/* ComputePlaneTangent, FunctionsSigmaProjection.h:68-88 */
static void plane_tangent(double *t, const orc_mc *m, double K, double G)
{
    const double sin_phi = m->sinphi, sin_psi = m->sinpsi;
    const double den = 6.0 * G + 2.0 * (G + 3.0 * K) * sin_phi * sin_psi;
    t[0] = (sin_phi - 1.0) * (-3.0 * G + (G + 3.0 * K) * sin_psi) / den;
    t[3] = (2.0 * G - 3.0 * K) * (sin_phi + 1.0) * sin_psi / den;
    t[6] = -(sin_phi + 1.0) * (-3.0 * G + (G + 3.0 * K) * sin_psi) / den;
    t[1] = 0.0;
    t[4] = 1.0;
    t[7] = 0.0;
    t[2] = -(sin_phi - 1.0) * (3.0 * G + (G + 3.0 * K) * sin_psi) / den;
    t[5] = (2.0 * G - 3.0 * K) * (sin_phi - 1.0) * sin_psi / den;
    t[8] = (sin_phi + 1.0) * (3.0 * G + (G + 3.0 * K) * sin_psi) / den;
}

/* ReturnMappingRightEdge, FunctionsSigmaProjection.h:93-158 */
static int rm_right_edge(const double *st, double *sp, double *hard, const orc_mc *m,
                         double K, double G)
{
    double ev[3] = {st[0], st[1], st[2]};
    const double sinphi = m->sinphi, sinpsi = m->sinpsi, cosphi = m->cosphi;
    const double c = m->cohesion;
    double gamma[2] = {0, 0}, phi[2], sb[2], ab[2], jac[2][2], ji[2][2];
    sb[0] = ev[0] - ev[2] + (ev[0] + ev[2]) * sinphi;
    sb[1] = ev[0] - ev[1] + (ev[0] + ev[1]) * sinphi;
    phi[0] = sb[0] - 2. * cosphi * c;
    phi[1] = sb[1] - 2. * cosphi * c;
    ab[0] = 4. * G * (1 + sinphi * sinpsi / 3.) + 4. * K * sinphi * sinpsi;
    ab[1] = 2. * G * (1. + sinphi + sinpsi - sinphi * sinpsi / 3.) + 4. * K * sinphi * sinpsi;
    for (int i = 0; i < 30; i++) {
        jac[0][0] = -ab[0];
        jac[1][0] = -ab[1];
        jac[0][1] = -ab[1];
        jac[1][1] = -ab[0];
        double det = jac[0][0] * jac[1][1] - jac[0][1] * jac[1][0];
        ji[0][0] = jac[1][1] / det;
        ji[1][0] = -jac[1][0] / det;
        ji[0][1] = -jac[0][1] / det;
        ji[1][1] = jac[0][0] / det;
        gamma[0] -= (ji[0][0] * phi[0] + ji[0][1] * phi[1]);
        gamma[1] -= (ji[1][0] * phi[0] + ji[1][1] * phi[1]);
        phi[0] = sb[0] - ab[0] * gamma[0] - ab[1] * gamma[1] - 2. * cosphi * c;
        phi[1] = sb[1] - ab[1] * gamma[0] - ab[0] * gamma[1] - 2. * cosphi * c;
        double res = (fabs(phi[0]) + fabs(phi[1]));
        if (fabs(res) < 1.e-12) break;
    }
    ev[0] -= (2. * G * (1 + sinpsi / 3.) + 2. * K * sinpsi) * (gamma[0] + gamma[1]);
    ev[1] += ((4. * G / 3. - K * 2.) * sinpsi) * gamma[0]
           + (2. * G * (1. - sinpsi / 3.) - 2. * K * sinpsi) * gamma[1];
    ev[2] += (2. * G * (1 - sinpsi / 3.) - 2. * K * sinpsi) * gamma[0]
           + ((4. * G / 3. - 2. * K) * sinpsi) * gamma[1];
    sp[0] = ev[0];
    sp[1] = ev[1];
    sp[2] = ev[2];
    *hard += (gamma[0] + gamma[1]) * 2. * cosphi;
    return (ev[0] > ev[1] || fabs(ev[0] - ev[1]) < 1.e-12) && (ev[1] > ev[2] || fabs(ev[1] - ev[2]) < 1.e-12);
}

/* ComputeRightEdgeTangent, FunctionsSigmaProjection.h:163-188 */
static void right_edge_tangent(double *t, const orc_mc *m, double K, double G)
{
    const double sin_phi = m->sinphi, sin_psi = m->sinpsi;
    const double a = 4.0 * G * (1.0 + (1.0 / 3.0) * sin_phi * sin_psi) + 4.0 * K * sin_phi * sin_psi;
    const double b = 2.0 * G * (1.0 + sin_phi + sin_psi - (1.0 / 3.0) * sin_phi * sin_psi) + 4.0 * K * sin_phi * sin_psi;
    t[0] = (3.0 * a + 3.0 * b - 4.0 * (1.0 + sin_phi) * (3.0 * K * sin_psi + G * (3.0 + sin_psi))) / (3. * (a + b));
    t[3] = (2.0 * (1.0 + sin_phi) * (-6.0 * K * sin_psi + G * (3.0 + sin_psi))) / (3. * (a + b));
    t[6] = (2.0 * (1.0 + sin_phi) * (-6.0 * K * sin_psi + G * (3.0 + sin_psi))) / (3. * (a + b));
    t[1] = (-2 * (-1 + sin_phi) * (3 * K * sin_psi + G * (3 + sin_psi))) / (3. * (a + b));
    t[4] = (-3 * b * b + 3 * a * (a + 2 * G * (-1 + sin_phi))
            - 2 * (a * G + 2 * b * G + 3 * a * K - 3 * b * K) * (-1 + sin_phi) * sin_psi) / (3. * (a - b) * (a + b));
    t[7] = (2 * (-1 + sin_phi) * (b * G * (-3 + sin_psi) + a * (2 * G - 3 * K) * sin_psi + 3 * b * K * sin_psi))
           / (3. * (a * a - b * b));
    t[2] = (-2 * (-1 + sin_phi) * (3 * K * sin_psi + G * (3 + sin_psi))) / (3. * (a + b));
    t[5] = (2 * (-1 + sin_phi) * (b * G * (-3 + sin_psi) + a * (2 * G - 3 * K) * sin_psi + 3 * b * K * sin_psi))
           / (3. * (a * a - b * b));
    t[8] = (-3 * b * b + 3 * a * (a + 2 * G * (-1 + sin_phi))
            - 2 * (a * G + 2 * b * G + 3 * a * K - 3 * b * K) * (-1 + sin_phi) * sin_psi) / (3. * (a - b) * (a + b));
}

/* ReturnMappingLeftEdge, FunctionsSigmaProjection.h:193-257 */
static int rm_left_edge(const double *st, double *sp, double *hard, const orc_mc *m,
                        double K, double G)
{
    double ev[3] = {st[0], st[1], st[2]};
    const double sinphi = m->sinphi, sinpsi = m->sinpsi, cosphi = m->cosphi;
    const double c = m->cohesion;
    const double sinphi2 = sinphi * sinphi;
    const double cosphi2 = 1. - sinphi2;
    double gamma[2] = {0, 0}, phi[2], sb[2], ab[2], jac[2][2], ji[2][2];
    sb[0] = ev[0] - ev[2] + (ev[0] + ev[2]) * sinphi;
    sb[1] = ev[1] - ev[2] + (ev[1] + ev[2]) * sinphi;
    ab[0] = 4. * G * (1 + sinphi * sinpsi / 3.) + 4. * K * sinphi * sinpsi;
    ab[1] = 2. * G * (1. - sinphi - sinpsi - sinphi * sinpsi / 3.) + 4. * K * sinphi * sinpsi;
    phi[0] = sb[0] - 2. * cosphi * c;
    phi[1] = sb[1] - 2. * cosphi * c;
    for (int i = 0; i < 30; i++) {
        jac[0][0] = -ab[0] - 4. * cosphi2 * 0;
        jac[1][0] = -ab[1] - 4. * cosphi2 * 0;
        jac[0][1] = -ab[1] - 4. * cosphi2 * 0;
        jac[1][1] = -ab[0] - 4. * cosphi2 * 0;
        double det = jac[0][0] * jac[1][1] - jac[0][1] * jac[1][0];
        ji[0][0] = jac[1][1] / det;
        ji[1][0] = -jac[1][0] / det;
        ji[0][1] = -jac[0][1] / det;
        ji[1][1] = jac[0][0] / det;
        gamma[0] -= (ji[0][0] * phi[0] + ji[0][1] * phi[1]);
        gamma[1] -= (ji[1][0] * phi[0] + ji[1][1] * phi[1]);
        phi[0] = sb[0] - ab[0] * gamma[0] - ab[1] * gamma[1] - 2. * cosphi * c;
        phi[1] = sb[1] - ab[1] * gamma[0] - ab[0] * gamma[1] - 2. * cosphi * c;
        double res = (fabs(phi[0]) + fabs(phi[1]));
        if (fabs(res) < 1.e-12) break;
    }
    ev[0] += -(2. * G * (1 + sinpsi / 3.) + 2. * K * sinpsi) * gamma[0]
           + ((4. * G / 3. - 2. * K) * sinpsi) * gamma[1];
    ev[1] += ((4. * G / 3. - K * 2.) * sinpsi) * gamma[0]
           - (2. * G * (1. + sinpsi / 3.) + 2. * K * sinpsi) * gamma[1];
    ev[2] += (2. * G * (1 - sinpsi / 3.) - 2. * K * sinpsi) * (gamma[0] + gamma[1]);
    sp[0] = ev[0];
    sp[1] = ev[1];
    sp[2] = ev[2];
    *hard += (gamma[0] + gamma[1]) * 2. * cosphi;
    return (ev[0] > ev[1] || fabs(ev[0] - ev[1]) < 1.e-12) && (ev[1] > ev[2] || fabs(ev[1] - ev[2]) < 1.e-12);
}

/* ComputeLeftEdgeTangent, FunctionsSigmaProjection.h:262-287 */
static void left_edge_tangent(double *t, const orc_mc *m, double K, double G)
{
    const double sin_phi = m->sinphi, sin_psi = m->sinpsi;
    const double a = 4.0 * G * (1.0 + (1.0 / 3.0) * sin_phi * sin_psi) + 4.0 * K * sin_phi * sin_psi;
    const double b = 2.0 * G * (1.0 - sin_phi - sin_psi - (1.0 / 3.0) * sin_phi * sin_psi) + 4.0 * K * sin_phi * sin_psi;
    t[0] = (-3 * b * b + 3 * a * (a - 2 * G * (1 + sin_phi))
            - 2 * (a * G + 2 * b * G + 3 * a * K - 3 * b * K) * (1 + sin_phi) * sin_psi) / (3. * (a - b) * (a + b));
    t[3] = (2 * (1 + sin_phi) * (a * (2 * G - 3 * K) * sin_psi + 3 * b * K * sin_psi + b * G * (3 + sin_psi)))
           / (3. * (a * a - b * b));
    t[6] = (-2 * (1 + sin_phi) * (G * (-3 + sin_psi) + 3 * K * sin_psi)) / (3. * (a + b));
    t[1] = (2 * (1 + sin_phi) * (a * (2 * G - 3 * K) * sin_psi + 3 * b * K * sin_psi + b * G * (3 + sin_psi)))
           / (3. * (a * a - b * b));
    t[4] = (-3 * b * b + 3 * a * (a - 2 * G * (1 + sin_phi))
            - 2 * (a * G + 2 * b * G + 3 * a * K - 3 * b * K) * (1 + sin_phi) * sin_psi) / (3. * (a - b) * (a + b));
    t[7] = (-2 * (1 + sin_phi) * (G * (-3 + sin_psi) + 3 * K * sin_psi)) / (3. * (a + b));
    t[2] = (2 * (-1 + sin_phi) * (G * (-3 + sin_psi) - 6 * K * sin_psi)) / (3. * (a + b));
    t[5] = (2 * (-1 + sin_phi) * (G * (-3 + sin_psi) - 6 * K * sin_psi)) / (3. * (a + b));
    t[8] = (3 * a + 3 * b - 4 * (-1 + sin_phi) * (G * (-3 + sin_psi) + 3 * K * sin_psi)) / (3. * (a + b));
}

/* ReturnMappingApex, FunctionsSigmaProjection.h:292-323 */
static void rm_apex(const double *st, double *sp, double *hard, const orc_mc *m, double K)
{
    const double cotphi = 1. / m->tanphi;
    double ptr = 0.;
    for (int i = 0; i < 3; i++) ptr += st[i];
    ptr /= 3.;
    double deps = 0.;
    double alpha = m->cosphi / m->sinpsi;
    double res = m->cohesion * cotphi - ptr;
    double p = 0.;
    for (int i = 0; i < 30; i++) {
        const double jac = K;   /* H = 0 */
        deps -= res / jac;
        p = ptr - K * deps;
        res = m->cohesion * cotphi - p;
        if (fabs(res) < 1.e-12) break;
    }
    *hard += alpha * deps;
    for (int i = 0; i < 3; i++) sp[i] = p;
}

/* ProjectSigma, FunctionsSigmaProjection.h:337-379 */
static void project_sigma(const double *ev, double *sp, int *mtype, double *alpha, const orc_mc *m,
                          double K, double G, double *grad, int want_grad)
{
    *mtype = 0;
    int ok = phi_plane(ev, sp, m);
    if (ok) {
        if (want_grad) {
            for (int i = 0; i < 9; i++) grad[i] = 0.;
            grad[0] = 1.;
            grad[4] = 1.;
            grad[8] = 1.;
        }
        return;
    }
    *mtype = 1;
    ok = rm_main_plane(ev, sp, alpha, m, K, G);
    if (ok && want_grad) plane_tangent(grad, m, K, G);
    if (!ok) {
        if (((1 - m->sinpsi) * ev[0] - 2. * ev[1] + (1 + m->sinpsi) * ev[2]) > 0) {
            ok = rm_right_edge(ev, sp, alpha, m, K, G);
            if (ok && want_grad) right_edge_tangent(grad, m, K, G);
        } else {
            ok = rm_left_edge(ev, sp, alpha, m, K, G);
            if (ok && want_grad) left_edge_tangent(grad, m, K, G);
        }
        if (!ok) {
            *mtype = -1;
            rm_apex(ev, sp, alpha, m, K);
            if (want_grad)
                for (int i = 0; i < 9; i++) grad[i] = 0;
        }
    }
}

/* ------------------------------------------- FunctionsTangentOperator.h */

/* Tangent variant for studies of the Newton iteration (the default, 0, is the
 * reference's arithmetic, which every parity test pins): 1 = the consistent
 * spectral tangent, with the spin factor of each eigen-pair from the
 * projected principal stresses and one ProdT pair per eigen-pair. */
static int g_consistent_tangent = 0;
void orc_set_consistent_tangent(int on) { g_consistent_tangent = on; }

/* TangentOperator, FunctionsTangentOperator.h:37-123 (6x6, row l, column k);
 * sp: the projected principal stresses (read by the consistent variant only) */
static void tangent_operator(const double *grad, const double *sev, const double *sp, const double *eev,
                             const double *evec, double *T, double G, double lambda)
{
    static const int ki_[6] = {0, 0, 0, 1, 1, 2};
    static const int kj_[6] = {0, 1, 2, 1, 2, 2};
    for (int l = 0; l < 36; ++l) T[l] = 0;
    for (int k = 0; k < 6; ++k) {
        const int ki = ki_[k], kj = kj_[k];
        for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 3; ++j) {
                double temp;
                if (ki == kj) {
                    temp = 2 * G * evec[j * 3 + kj] * evec[j * 3 + ki];
                    temp += lambda;
                } else {
                    temp = 2 * G * evec[j * 3 + kj] * evec[j * 3 + ki];
                    temp *= 2.;
                }
                for (int l = 0; l < 6; ++l) {
                    const int li = ki_[l], lj = kj_[l];
                    T[l * 6 + k] += temp * grad[i * 3 + j] * evec[i * 3 + li] * evec[i * 3 + lj];
                }
            }
        }
    }
    double tempMat[9], tmp[9], col[6];
    for (int i = 0; i < 9; i++) tempMat[i] = 0;
    for (int i = 0; i < 2; ++i) {
        for (int j = i + 1; j < 3; ++j) {
            double deps = eev[i] - eev[j];
            double dsig = g_consistent_tangent ? sp[i] - sp[j] : sev[i] - sev[j];
            if (g_consistent_tangent)
                for (int q = 0; q < 9; q++) tempMat[q] = 0;
            double factor = 0.;
            if (!((fabs(deps) < 1.e-12) || (deps < 0.0)))
                factor = dsig / deps;
            else
                factor = G * (grad[i * 3 + i] - grad[i * 3 + j] - grad[j * 3 + i] + grad[j * 3 + j]);
            /* ProdT(v_i, v_j) and ProdT(v_j, v_i) accumulate into tempMat,
             * which is not reset between pairs (…h:75, 90-102) */
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) tempMat[a * 3 + b] += evec[3 * i + a] * evec[3 * j + b];
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) tempMat[a * 3 + b] += evec[3 * j + a] * evec[3 * i + b];
            for (int k = 0; k < 6; ++k) {
                const int ki = ki_[k], kj = kj_[k];
                double val;
                if (ki == kj)
                    val = evec[j * 3 + ki] * evec[i * 3 + kj] * factor;
                else
                    val = (evec[j * 3 + ki] * evec[i * 3 + kj] + evec[j * 3 + kj] * evec[i * 3 + ki]) * factor;
                for (int q = 0; q < 9; q++) tmp[q] = val * tempMat[q];
                int c = 0;
                for (int a = 0; a < 3; a++)
                    for (int b = a; b < 3; b++) col[c++] = tmp[a * 3 + b];
                for (int l = 0; l < 6; l++) {
                    double aux = T[l * 6 + k];
                    T[l * 6 + k] = aux + col[l];
                }
            }
        }
    }
}

/* ----------------------------------------- full tangent (verification) */

/* The point update of orc_ip_update with the full 6x6 tangent T (row l =
 * stress component, column k = strain component, order XX XY XZ YY YZ ZZ)
 * instead of its plane-strain extraction: what TPZPlasticStepPV::
 * ApplyStrainComputeSigma returns as Dep and TRKSolution::RKProcess reads
 * (TRKSolution.cpp:189-191).  strain6 is the total strain (tensor shear). */
/* SpectralDecomposition of one symmetric tensor (XX XY XZ YY YZ ZZ), for
 * tests of the decomposition itself */
void orc_spectral(const double s6[6], double ev[3], double vec9[9])
{
    double s[6];
    for (int i = 0; i < 6; i++) s[i] = s6[i];
    spectral(s, ev, vec9);
}

void orc_ip_tangent6(const orc_elastic *el, const orc_mc *mc, const double strain6_in[6], const double eps_p6[6],
                     double sigma6[6], double eps_p6_out[6], double T36[36], int *mtype)
{
    const double lambda = el->lambda, mu = el->mu;
    const double G = mu;
    const double K = lambda + 2 * mu / 3;
    double strain[6], ee[6], sig[6], pl[6];
    double sev[3], svec[9], sp[3], grad[9], eev[3], evec[9];
    double a = 0.0;
    int mt = 0;
    for (int i = 0; i < 6; i++) {
        strain[i] = strain6_in[i];
        pl[i] = eps_p6[i];
    }
    elastic_strain(pl, strain, ee);
    trial_stress(ee, sig, mu, lambda);
    spectral(sig, sev, svec);
    ee[1] = ee[1] / 2;
    spectral(ee, eev, evec);
    project_sigma(sev, sp, &mt, &a, mc, K, G, grad, 1);
    tangent_operator(grad, sev, sp, eev, evec, T36, G, lambda);
    reconstruct(sp, svec, sig);
    strain_from_stress(sig, ee, mu, lambda);
    plastic_strain(strain, ee, pl);
    for (int i = 0; i < 6; i++) {
        sigma6[i] = sig[i];
        eps_p6_out[i] = pl[i];
    }
    if (mtype) *mtype = mt;
}

/* -------------------------------------------------- per-point update */

void orc_ip_update(const orc_elastic *el, const orc_mc *mc,
                   const double strain3[3], const double eps_p6[6], double weight,
                   double sigma_w3[3], double *dep9,
                   double sigma6[6], double eps_p6_out[6], double strain6[6],
                   int *mtype, double *alpha)
{
    const double lambda = el->lambda, mu = el->mu;
    const double G = mu;
    const double K = lambda + 2 * mu / 3;
    double strain[6], ee[6], sig[6], pl[6];
    double sev[3], svec[9], sp[3], grad[9];
    double a = 0.0;
    int mt = 0;

    compose_strain(strain3, strain);
    for (int i = 0; i < 6; i++) pl[i] = eps_p6[i];
    elastic_strain(pl, strain, ee);
    trial_stress(ee, sig, mu, lambda);
    spectral(sig, sev, svec);
    if (dep9) {
        double eev[3], evec[9], T[36];
        ee[1] = ee[1] / 2;
        spectral(ee, eev, evec);
        project_sigma(sev, sp, &mt, &a, mc, K, G, grad, 1);
        tangent_operator(grad, sev, sp, eev, evec, T, G, lambda);
        reconstruct(sp, svec, sig);
        strain_from_stress(sig, ee, mu, lambda);
        plastic_strain(strain, ee, pl);
        translate_dep(T, grad);
        for (int i = 0; i < 9; i++) dep9[i] = grad[i] * weight;
    } else {
        project_sigma(sev, sp, &mt, &a, mc, K, G, grad, 0);
        reconstruct(sp, svec, sig);
        strain_from_stress(sig, ee, mu, lambda);
        plastic_strain(strain, ee, pl);
    }
    sigma_w3[0] = sig[XX] * weight;
    sigma_w3[1] = sig[XY] * weight;
    sigma_w3[2] = sig[YY] * weight;
    if (sigma6) memcpy(sigma6, sig, sizeof sig);
    if (eps_p6_out) memcpy(eps_p6_out, pl, sizeof pl);
    if (strain6) memcpy(strain6, strain, sizeof strain);
    *mtype = mt;
    *alpha = a;
}

void orc_ip_update_gpu_alias(const orc_elastic *el, const orc_mc *mc,
                             const double strain3[3], const double eps_p6[6], double weight,
                             double sigma_w3[3], double sigma6[6], double eps_p6_out[6],
                             int *mtype, double *alpha)
{
    const double lambda = el->lambda, mu = el->mu;
    const double G = mu;
    const double K = lambda + 2 * mu / 3;
    double strain[6], ee[6], sig[6], pl[6], svec[9], sp[3], grad[9];
    double a = 0.0;
    int mt = 0;
    compose_strain(strain3, strain);
    for (int i = 0; i < 6; i++) pl[i] = eps_p6[i];
    elastic_strain(pl, strain, ee);
    trial_stress(ee, sig, mu, lambda);
    spectral(sig, sp, svec);
    project_sigma(sp, sp, &mt, &a, mc, K, G, grad, 0);   /* input aliases output */
    reconstruct(sp, svec, sig);
    strain_from_stress(sig, ee, mu, lambda);
    plastic_strain(strain, ee, pl);
    sigma_w3[0] = weight * sig[XX];
    sigma_w3[1] = weight * sig[XY];
    sigma_w3[2] = weight * sig[YY];
    if (sigma6) memcpy(sigma6, sig, sizeof sig);
    if (eps_p6_out) memcpy(eps_p6_out, pl, sizeof pl);
    *mtype = mt;
    *alpha = a;
}

void orc_compute_sigma_batch(int64_t npts, int pts_per_mat,
                             const orc_elastic *el, const orc_mc *mats,
                             const double *strain3, double *eps_p6,
                             const double *weight, int update_mem,
                             double *sigma_w3, double *dep9,
                             double *sigma6_state, int8_t *mtype, double *alpha)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < npts; i++) {
        double s6[6], p6[6];
        int mt;
        double a;
        orc_ip_update(el, &mats[i / pts_per_mat], &strain3[3 * i], &eps_p6[6 * i], weight[i],
                      &sigma_w3[3 * i], dep9 ? &dep9[9 * i] : 0, s6, p6, 0, &mt, &a);
        if (update_mem) {
            for (int k = 0; k < 6; k++) eps_p6[6 * i + k] = p6[k];
            if (sigma6_state)
                for (int k = 0; k < 6; k++) sigma6_state[6 * i + k] = s6[k];
            if (mtype) mtype[i] = (int8_t)mt;
            if (alpha) alpha[i] = a;
        }
    }
}
