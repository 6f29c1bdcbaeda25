// Per-integration-point Mohr-Coulomb update on the device (FP64).
//
// Plane-strain form of the reference's constitutive sequence
// (TPZConstitutiveLawProcessor.cpp:163-195 / 377-423 with FunctionsStressStrain.h,
// FunctionsSpectralDecomp.h, FunctionsSigmaProjection.h, FunctionsTangentOperator.h).
// In plane strain the XZ and YZ components of strain, plastic strain and
// stress are exactly zero, so tensors carry four components (xx, xy, yy, zz)
// and every term that multiplies a structural zero is dropped.  All remaining
// operations keep the reference's association and order, and the translation
// unit is compiled with --fmad=false, so each result equals the reference CPU
// arithmetic bit for bit (up to the sign of an exact zero).
//
// Undefined behaviour of the reference is given the oracle's meaning:
// gamma[2] of the edge returns starts at 0, alpha accumulates from 0, abs()
// of the cubic residual is fabs().
#pragma once

// The same source compiles for the host (g++, -ffp-contract=off), where a CPU
// test compares it with the oracle bit for bit.
#if defined(__CUDACC__)
#define IPFEM_HD __host__ __device__ __forceinline__
#else
#include <cmath>
#define IPFEM_HD inline
using std::fabs;
using std::sqrt;
#endif

struct MCConst {            // per-element Mohr-Coulomb constants (libm trig from the host)
    double c, sinphi, cosphi, tanphi, sinpsi;
};

struct ElasticConst {
    double lambda, mu;
    double K, G;            // lambda + 2 mu / 3, mu
    double l2m;             // lambda + 2 * mu
    double c1, c2, inv_mu;  // inverse elasticity coefficients of ComputeStrain
    int consistent;         // 1: consistent spectral tangent (ipfem_set_consistent_tangent)
    int spectral;           // 1: closed-form plane-strain decomposition (ipfem_set_spectral_mode)
};

// ------------------------------------------------ spectral decomposition
// Symmetric 3x3 with s_xz = s_yz = 0.  s = {xx, xy, yy, zz}.
// FunctionsSpectralDecomp.h:61-111 (Newton on the normalised cubic)
IPFEM_HD void sd_newton(const double s[4], double ev[3], double maxel)
{
    const double sxx = s[0], sxy = s[1], syy = s[2], szz = s[3];
    const double sxy2 = sxy * sxy;
    const double P = sxx * syy, Q = sxx * szz, R = syy * szz;
    const double t2 = sxy2 * szz;
    const double t5 = P * szz;
    const double tr = (sxx + syy) + szz;
    const double I2 = ((sxy2 - P) - Q) - R;
    const double dc = ((sxy2 - P) - Q) - R;   // df constant part, same sequence
#pragma unroll 1
    for (int i = 0; i < 2; i++) {
        double x;
        if (i == 0) {
            // Interval, FunctionsSpectralDecomp.h:25-56 (upper bound)
            const double a = fabs(sxy);
            double up = sxx + a;
            const double u1 = syy + a, u2 = szz + a;
            if (u1 > up) up = u1;
            if (u2 > up) up = u2;
            x = up;
        } else {
            const double a = fabs(sxy);
            double lo = sxx - a;
            const double l1 = syy - a, l2 = szz - a;
            if (l1 < lo) lo = l1;
            if (l2 < lo) lo = l2;
            x = lo;
        }
        double f = ((((-x * x * x - t2) + t5) + x * x * tr) + x * I2);
        double res = fabs(f);
        int it = 0;
#pragma unroll 1
        while (it < 20 && res > 10e-12) {
            const double df = ((-3 * x * x + sxy2) - P - Q - R) + 2 * x * tr;
            x -= f / df;
            f = ((((-x * x * x - t2) + t5) + x * x * tr) + x * I2);
            res = fabs(f);
            it++;
        }
        ev[i] = x;
    }
    (void)dc;
    ev[2] = tr - ev[0] - ev[1];
    ev[0] *= maxel;
    ev[1] *= maxel;
    ev[2] *= maxel;
    // descending sort, FunctionsSpectralDecomp.h:100-110
    if (ev[0] < ev[1]) { double a = ev[0]; ev[0] = ev[1]; ev[1] = a; }
    if (ev[0] < ev[2]) { double a = ev[0]; ev[0] = ev[2]; ev[2] = a; }
    if (ev[1] < ev[2]) { double a = ev[1]; ev[1] = ev[2]; ev[2] = a; }
}

// Multiplicity1, FunctionsSpectralDecomp.h:116-150
IPFEM_HD void sd_mult1(const double s[4], double lam, double *v_out)
{
    const double sxx = s[0], sxy = s[1], syy = s[2], szz = s[3];
    const double det0 = (sxx - lam) * (syy - lam) - sxy * sxy;
    const double det1 = (sxx - lam) * (szz - lam);
    const double det2 = (syy - lam) * (szz - lam);
    double maxdet = fabs(det0);
    if (fabs(det1) > fabs(maxdet)) maxdet = fabs(det1);
    if (fabs(det2) > fabs(maxdet)) maxdet = fabs(det2);
    double v0, v1, v2;
    if (maxdet == fabs(det0)) {
        const double r = 1 / det0;
        v0 = r * 0.0;
        v1 = r * 0.0;
        v2 = 1;
    } else if (maxdet == fabs(det1)) {
        const double r = 1 / det1;
        v0 = r * (-(szz - lam) * sxy);
        v1 = 1;
        v2 = r * 0.0;
    } else {
        const double r = 1 / det2;
        v0 = 1;
        v1 = r * (-(szz - lam) * sxy);
        v2 = r * 0.0;
    }
    const double norm = sqrt(v0 * v0 + v1 * v1 + v2 * v2);
    v_out[0] = v0 / norm;
    v_out[1] = v1 / norm;
    v_out[2] = v2 / norm;
}

// Multiplicity2, FunctionsSpectralDecomp.h:155-212 (second norm as in the reference)
IPFEM_HD void sd_mult2(const double s[4], double lam, double *a, double *b)
{
    const double x0 = s[0] - lam, x1 = s[2] - lam, x2 = s[3] - lam;
    double maxx = fabs(x0);
    if (fabs(x1) > fabs(maxx)) maxx = fabs(x1);
    if (fabs(x2) > fabs(maxx)) maxx = fabs(x2);
    double v1[3], v2[3];
    if (maxx == fabs(x0)) {
        v1[0] = -s[1] / x0; v1[1] = 1; v1[2] = 0;
        v2[0] = -0.0 / x0;  v2[1] = 0; v2[2] = 1;
    } else if (maxx == fabs(x1)) {
        v1[0] = 1; v1[1] = -s[1] / x1; v1[2] = 0;
        v2[0] = 0; v2[1] = -0.0 / x1;  v2[2] = 1;
    } else {
        v1[0] = 1; v1[1] = 0; v1[2] = -0.0 / x2;
        v2[0] = 0; v2[1] = 1; v2[2] = -0.0 / x2;
    }
    const double n1 = sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
    const double n2 = sqrt(v2[0] * v2[0] + v2[1] * v1[1] + v2[2] * v2[2]);
    a[0] = v1[0] / n1; a[1] = v1[1] / n1; a[2] = v1[2] / n1;
    b[0] = v2[0] / n2; b[1] = v2[1] / n2; b[2] = v2[2] / n2;
}

// SpectralDecomposition, FunctionsSpectralDecomp.h:261-268.  s is modified
// (normalised and rescaled) exactly as the reference modifies its argument.
IPFEM_HD void spectral(double s[4], double ev[3], double vec[9])
{
    // Normalize (…h:7-20); XZ and YZ are zero and never exceed |maxel|
    double m = s[0];
    if (fabs(s[1]) > fabs(m)) m = s[1];
    if (fabs(s[2]) > fabs(m)) m = s[2];
    if (fabs(s[3]) > fabs(m)) m = s[3];
    if (m != 0) {
        s[0] /= m; s[1] /= m; s[2] /= m; s[3] /= m;
    }
    sd_newton(s, ev, m);
    // Eigenvectors (…h:217-256)
    s[0] *= m; s[1] *= m; s[2] *= m; s[3] *= m;
    if ((ev[0] == ev[1]) && (ev[1] == ev[2])) {
        vec[0] = 1.; vec[1] = 0.; vec[2] = 0.;
        vec[3] = 0.; vec[4] = 1.; vec[5] = 0.;
        vec[6] = 0.; vec[7] = 0.; vec[8] = 1.;
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

// Closed-form decomposition of a plane-strain tensor s = {xx, xy, yy, zz}:
// zz with (0, 0, 1), and the eigen-pairs of the in-plane 2x2 block, so the
// vectors are orthonormal at any eigenvalue gap (the decomposition above loses
// that within about 1e-6, relative, of a repeated eigenvalue: its cubic roots
// are about 3e-6 off there and Multiplicity1 can return the same vector
// twice).  Same outputs as spectral(): eigenvalues descending, vectors as rows.
IPFEM_HD void spectral_plane(const double s[4], double ev[3], double vec[9])
{
    const double d = 0.5 * (s[0] - s[2]), m = 0.5 * (s[0] + s[2]);
    const double r = sqrt(d * d + s[1] * s[1]);
    double c = 1.0, sn = 0.0;       // unit eigenvector of m + r
    if (r > 0.0) {
        // (A - (m + r) I) x = 0 for x = (d + r, b) and for x = (b, r - d):
        // take the one with an entry of at least r
        const double x = d >= 0.0 ? d + r : s[1];
        const double y = d >= 0.0 ? s[1] : r - d;
        const double n = sqrt(x * x + y * y);
        c = x / n;
        sn = y / n;
    }
    const double l0 = m + r, l1 = m - r, l2 = s[3];
    // descending; m + r >= m - r, and zz goes after an equal in-plane value
    double e0 = l0, e1 = l1, e2 = l2;
    double v0[3] = {c, sn, 0.0}, v1[3] = {-sn, c, 0.0}, v2[3] = {0.0, 0.0, 1.0};
    if (l2 > l0) {
        e0 = l2; e1 = l0; e2 = l1;
        v0[0] = 0.0; v0[1] = 0.0; v0[2] = 1.0;
        v1[0] = c; v1[1] = sn; v1[2] = 0.0;
        v2[0] = -sn; v2[1] = c; v2[2] = 0.0;
    } else if (l2 > l1) {
        e1 = l2; e2 = l1;
        v1[0] = 0.0; v1[1] = 0.0; v1[2] = 1.0;
        v2[0] = -sn; v2[1] = c; v2[2] = 0.0;
    }
    ev[0] = e0; ev[1] = e1; ev[2] = e2;
    vec[0] = v0[0]; vec[1] = v0[1]; vec[2] = v0[2];
    vec[3] = v1[0]; vec[4] = v1[1]; vec[5] = v1[2];
    vec[6] = v2[0]; vec[7] = v2[1]; vec[8] = v2[2];
}

// ----------------------------------------------------- Mohr-Coulomb return
// FunctionsSigmaProjection.h:6-20
IPFEM_HD bool phi_plane(const double ev[3], const MCConst &m)
{
    const double phi = ev[0] - ev[2] + (ev[0] + ev[2]) * m.sinphi - 2. * m.c * m.cosphi;
    return (fabs(phi) < 1.e-12) || (phi < 0.0);
}

// FunctionsSigmaProjection.h:25-63
IPFEM_HD bool rm_main_plane(const double st[3], double sp[3], double &hard,
                                              const MCConst &m, double K, double G)
{
    double e0 = st[0], e1 = st[1], e2 = st[2];
    const double sinphi = m.sinphi, sinpsi = m.sinpsi, cosphi = m.cosphi;
    const double constA = 4. * G * (1. + sinphi * sinpsi / 3.) + 4. * K * sinphi * sinpsi;
    const double b = e0 - e2 + (e0 + e2) * sinphi - 2. * m.c * cosphi;
    double phi = b;
    double gamma = 0;
    const double jac = -constA;          // -constA - 4*cos^2(phi)*H, H = 0
#pragma unroll 1
    for (int i = 0; i < 30; i++) {
        const double dgamma = -phi / jac;
        gamma += dgamma;
        phi = b - constA * gamma;
        if (fabs(phi) < 1.e-12) break;
    }
    e0 -= (2. * G * (1 + sinpsi / 3.) + 2. * K * sinpsi) * gamma;
    e1 += (4. * G / 3. - K * 2.) * sinpsi * gamma;
    e2 += (2. * G * (1 - sinpsi / 3.) - 2. * K * sinpsi) * gamma;
    sp[0] = e0; sp[1] = e1; sp[2] = e2;
    hard += gamma * 2. * cosphi;
    return (e0 > e1 || fabs(e0 - e1) < 1.e-12) && (e1 > e2 || fabs(e1 - e2) < 1.e-12);
}

// FunctionsSigmaProjection.h:68-88
IPFEM_HD void plane_tangent(double t[9], const MCConst &m, double K, double G)
{
    const double sin_phi = m.sinphi, sin_psi = m.sinpsi;
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

// Two-surface return on an edge (FunctionsSigmaProjection.h:93-158 right,
// 193-257 left).  The Jacobian is loop-invariant with H = 0.
template <bool RIGHT>
IPFEM_HD bool rm_edge(const double st[3], double sp[3], double &hard,
                                        const MCConst &m, double K, double G)
{
    double e0 = st[0], e1 = st[1], e2 = st[2];
    const double sinphi = m.sinphi, sinpsi = m.sinpsi, cosphi = m.cosphi, c = m.c;
    double g0 = 0, g1 = 0, sb0, sb1, ab0, ab1;
    sb0 = e0 - e2 + (e0 + e2) * sinphi;
    if (RIGHT) sb1 = e0 - e1 + (e0 + e1) * sinphi;
    else       sb1 = e1 - e2 + (e1 + e2) * sinphi;
    ab0 = 4. * G * (1 + sinphi * sinpsi / 3.) + 4. * K * sinphi * sinpsi;
    if (RIGHT) ab1 = 2. * G * (1. + sinphi + sinpsi - sinphi * sinpsi / 3.) + 4. * K * sinphi * sinpsi;
    else       ab1 = 2. * G * (1. - sinphi - sinpsi - sinphi * sinpsi / 3.) + 4. * K * sinphi * sinpsi;
    const double cc = 2. * cosphi * c;
    double phi0 = sb0 - cc;
    double phi1 = sb1 - cc;
    const double j00 = -ab0, j10 = -ab1, j01 = -ab1, j11 = -ab0;
    const double det = j00 * j11 - j01 * j10;
    const double i00 = j11 / det, i10 = -j10 / det, i01 = -j01 / det, i11 = j00 / det;
#pragma unroll 1
    for (int i = 0; i < 30; i++) {
        g0 -= (i00 * phi0 + i01 * phi1);
        g1 -= (i10 * phi0 + i11 * phi1);
        phi0 = sb0 - ab0 * g0 - ab1 * g1 - cc;
        phi1 = sb1 - ab1 * g0 - ab0 * g1 - cc;
        const double res = (fabs(phi0) + fabs(phi1));
        if (fabs(res) < 1.e-12) break;
    }
    if (RIGHT) {
        e0 -= (2. * G * (1 + sinpsi / 3.) + 2. * K * sinpsi) * (g0 + g1);
        e1 += ((4. * G / 3. - K * 2.) * sinpsi) * g0 + (2. * G * (1. - sinpsi / 3.) - 2. * K * sinpsi) * g1;
        e2 += (2. * G * (1 - sinpsi / 3.) - 2. * K * sinpsi) * g0 + ((4. * G / 3. - 2. * K) * sinpsi) * g1;
    } else {
        e0 += -(2. * G * (1 + sinpsi / 3.) + 2. * K * sinpsi) * g0 + ((4. * G / 3. - 2. * K) * sinpsi) * g1;
        e1 += ((4. * G / 3. - K * 2.) * sinpsi) * g0 - (2. * G * (1. + sinpsi / 3.) + 2. * K * sinpsi) * g1;
        e2 += (2. * G * (1 - sinpsi / 3.) - 2. * K * sinpsi) * (g0 + g1);
    }
    sp[0] = e0; sp[1] = e1; sp[2] = e2;
    hard += (g0 + g1) * 2. * cosphi;
    return (e0 > e1 || fabs(e0 - e1) < 1.e-12) && (e1 > e2 || fabs(e1 - e2) < 1.e-12);
}

// FunctionsSigmaProjection.h:163-188
IPFEM_HD void right_edge_tangent(double t[9], const MCConst &m, double K, double G)
{
    const double sin_phi = m.sinphi, sin_psi = m.sinpsi;
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

// FunctionsSigmaProjection.h:262-287
IPFEM_HD void left_edge_tangent(double t[9], const MCConst &m, double K, double G)
{
    const double sin_phi = m.sinphi, sin_psi = m.sinpsi;
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

// FunctionsSigmaProjection.h:292-323
IPFEM_HD void rm_apex(const double st[3], double sp[3], double &hard,
                                        const MCConst &m, double K)
{
    const double cotphi = 1. / m.tanphi;
    double ptr = 0.;
    ptr += st[0];
    ptr += st[1];
    ptr += st[2];
    ptr /= 3.;
    double deps = 0.;
    const double alpha = m.cosphi / m.sinpsi;
    const double ccot = m.c * cotphi;
    double res = ccot - ptr;
    double p = 0.;
#pragma unroll 1
    for (int i = 0; i < 30; i++) {
        deps -= res / K;
        p = ptr - K * deps;
        res = ccot - p;
        if (fabs(res) < 1.e-12) break;
    }
    hard += alpha * deps;
    sp[0] = p; sp[1] = p; sp[2] = p;
}

// ProjectSigma, FunctionsSigmaProjection.h:337-379 (separate input/output
// arrays as in the CPU path, TPZConstitutiveLawProcessor.cpp:184)
template <bool GRAD>
IPFEM_HD int project_sigma(const double ev[3], double sp[3], double &alpha,
                                             const MCConst &m, double K, double G, double grad[9])
{
    sp[0] = ev[0]; sp[1] = ev[1]; sp[2] = ev[2];
    if (phi_plane(ev, m)) {
        if (GRAD) {
#pragma unroll
            for (int i = 0; i < 9; i++) grad[i] = 0.;
            grad[0] = 1.; grad[4] = 1.; grad[8] = 1.;
        }
        return 0;
    }
    bool ok = rm_main_plane(ev, sp, alpha, m, K, G);
    if (ok) {
        if (GRAD) plane_tangent(grad, m, K, G);
        return 1;
    }
    if (((1 - m.sinpsi) * ev[0] - 2. * ev[1] + (1 + m.sinpsi) * ev[2]) > 0) {
        ok = rm_edge<true>(ev, sp, alpha, m, K, G);
        if (ok && GRAD) right_edge_tangent(grad, m, K, G);
    } else {
        ok = rm_edge<false>(ev, sp, alpha, m, K, G);
        if (ok && GRAD) left_edge_tangent(grad, m, K, G);
    }
    if (ok) return 1;
    rm_apex(ev, sp, alpha, m, K);
    if (GRAD) {
#pragma unroll
        for (int i = 0; i < 9; i++) grad[i] = 0;
    }
    return -1;
}

// ------------------------------------------------------- tangent operator
// TangentOperator (FunctionsTangentOperator.h:37-123) restricted to the
// entries that TranslateDep keeps (rows and columns XX, XY, YY = Voigt 0, 1, 3),
// then TranslateDep (FunctionsStressStrain.h:103-119).  Each kept entry is
// accumulated in the reference's order.  With consistent = 1 the spin factor
// of each eigen-pair takes the projected principal stresses sp instead of the
// trial ones and the pair's ProdT terms start from zero: the consistent
// spectral tangent (the reference's differs from finite differences of its
// own residual by about 1e-2 in plastic states).
IPFEM_HD void tangent_dep(const double grad[9], const double sev[3], const double sp[3],
                                            const double eev[3], const double v[9], double G, double lambda,
                                            int consistent, double dep[9])
{
    // Voigt k -> (ki, kj): 0 -> (0,0), 1 -> (0,1), 3 -> (1,1)
    double T[3][3];     // T[l][k] over l, k in {XX, XY, YY}
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int b = 0; b < 3; b++) T[a][b] = 0;
#pragma unroll
    for (int kk = 0; kk < 3; kk++) {
        const int ki = (kk == 2) ? 1 : 0;
        const int kj = (kk == 0) ? 0 : 1;
#pragma unroll
        for (int i = 0; i < 3; i++) {
#pragma unroll
            for (int j = 0; j < 3; j++) {
                double temp;
                if (ki == kj) {
                    temp = 2 * G * v[j * 3 + kj] * v[j * 3 + ki];
                    temp += lambda;
                } else {
                    temp = 2 * G * v[j * 3 + kj] * v[j * 3 + ki];
                    temp *= 2.;
                }
                const double tg = temp * grad[i * 3 + j];
                T[0][kk] += tg * v[i * 3 + 0] * v[i * 3 + 0];
                T[1][kk] += tg * v[i * 3 + 0] * v[i * 3 + 1];
                T[2][kk] += tg * v[i * 3 + 1] * v[i * 3 + 1];
            }
        }
    }
    double tm00 = 0, tm01 = 0, tm11 = 0;   // tempMat entries (0,0), (0,1), (1,1)
#pragma unroll
    for (int pr = 0; pr < 3; pr++) {
        const int i = (pr == 2) ? 1 : 0;
        const int j = (pr == 0) ? 1 : 2;
        const double deps = eev[i] - eev[j];
        const double dsig = consistent ? sp[i] - sp[j] : sev[i] - sev[j];
        if (consistent) {
            tm00 = 0;
            tm01 = 0;
            tm11 = 0;
        }
        double factor = 0.;
        if (!((fabs(deps) < 1.e-12) || (deps < 0.0)))
            factor = dsig / deps;
        else
            factor = G * (grad[i * 3 + i] - grad[i * 3 + j] - grad[j * 3 + i] + grad[j * 3 + j]);
        tm00 += v[3 * i + 0] * v[3 * j + 0];
        tm01 += v[3 * i + 0] * v[3 * j + 1];
        tm11 += v[3 * i + 1] * v[3 * j + 1];
        tm00 += v[3 * j + 0] * v[3 * i + 0];
        tm01 += v[3 * j + 0] * v[3 * i + 1];
        tm11 += v[3 * j + 1] * v[3 * i + 1];
#pragma unroll
        for (int kk = 0; kk < 3; kk++) {
            const int ki = (kk == 2) ? 1 : 0;
            const int kj = (kk == 0) ? 0 : 1;
            double val;
            if (ki == kj)
                val = v[j * 3 + ki] * v[i * 3 + kj] * factor;
            else
                val = (v[j * 3 + ki] * v[i * 3 + kj] + v[j * 3 + kj] * v[i * 3 + ki]) * factor;
            T[0][kk] = T[0][kk] + val * tm00;
            T[1][kk] = T[1][kk] + val * tm01;
            T[2][kk] = T[2][kk] + val * tm11;
        }
    }
#pragma unroll
    for (int a = 0; a < 3; a++) {
        dep[3 * a + 0] = T[a][0];
        dep[3 * a + 1] = T[a][1] / 2;
        dep[3 * a + 2] = T[a][2];
    }
}

// ----------------------------------------------------------- point update
// One integration point.  eps = (eps_xx, gamma_xy, eps_yy) = B u; pl = committed
// plastic strain {xx, xy, yy, zz}.  Outputs the stress {xx, xy, yy, zz}, the
// updated plastic strain, alpha, m_type and, if DEP, the unweighted 3x3 Dep.
template <bool DEP>
IPFEM_HD int ip_update(const double eps[3], const double pl[4], const ElasticConst &E,
                                         const MCConst &m, double sig[4], double pl_out[4],
                                         double &alpha, double dep[9])
{
    // ComposeStrain + ElasticStrain (FunctionsStressStrain.h:10-33)
    double ee[4];
    ee[0] = eps[0] - pl[0];
    ee[1] = eps[1] - pl[1];
    ee[2] = eps[2] - pl[2];
    ee[3] = 0.0 - pl[3];
    // ComputeTrialStress (…h:47-55)
    double s[4];
    s[0] = E.l2m * ee[0] + E.lambda * ee[2] + E.lambda * ee[3];
    s[2] = E.lambda * ee[0] + E.l2m * ee[2] + E.lambda * ee[3];
    s[3] = E.lambda * ee[0] + E.lambda * ee[2] + E.l2m * ee[3];
    s[1] = E.mu * ee[1];
    double sev[3], svec[9], sp[3], grad[9];
    if (E.spectral == 1)
        spectral_plane(s, sev, svec);
    else
        spectral(s, sev, svec);
    alpha = 0.0;
    int mt;
    if (DEP) {
        double eev[3], evec[9];
        ee[1] = ee[1] / 2;
        if (E.spectral == 1)
            spectral_plane(ee, eev, evec);
        else
            spectral(ee, eev, evec);
        mt = project_sigma<true>(sev, sp, alpha, m, E.K, E.G, grad);
        tangent_dep(grad, sev, sp, eev, evec, E.G, E.lambda, E.consistent, dep);
    } else {
        mt = project_sigma<false>(sev, sp, alpha, m, E.K, E.G, grad);
    }
    // ReconstructStressTensor (…h:60-68)
    sig[0] = (sp[0] * svec[0] * svec[0] + sp[1] * svec[3] * svec[3] + sp[2] * svec[6] * svec[6]);
    sig[2] = (sp[0] * svec[1] * svec[1] + sp[1] * svec[4] * svec[4] + sp[2] * svec[7] * svec[7]);
    sig[3] = (sp[0] * svec[2] * svec[2] + sp[1] * svec[5] * svec[5] + sp[2] * svec[8] * svec[8]);
    sig[1] = (sp[0] * svec[0] * svec[1] + sp[1] * svec[3] * svec[4] + sp[2] * svec[6] * svec[7]);
    // ComputeStrain + PlasticStrain (…h:38-42, 73-81)
    const double exx = E.c1 * sig[0] - E.c2 * (sig[2] + sig[3]);
    const double eyy = E.c1 * sig[2] - E.c2 * (sig[0] + sig[3]);
    const double ezz = E.c1 * sig[3] - E.c2 * (sig[2] + sig[0]);
    const double exy = E.inv_mu * sig[1];
    pl_out[0] = eps[0] - exx;
    pl_out[1] = eps[1] - exy;
    pl_out[2] = eps[2] - eyy;
    pl_out[3] = 0.0 - ezz;
    return mt;
}
