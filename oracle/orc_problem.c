/*
 * CPU oracle (test infrastructure only): wellbore problem, setup, residual
 * and tangent assembly, Jacobi-PCG and the load-stepped Newton loop.
 *
 * Reference correspondence (labmec/IntPointsFEM):
 *   orc_element_blocks   TPZNumericalIntegrator.cpp:272-388 (B blocks, row-major
 *                        (3*npts) x (2*nshape), row order [eps_xx, gamma_xy, eps_yy])
 *                        and :420-427 (weights w*|detJ|)
 *   dof map              TPZNumericalIntegrator.cpp:429-443
 *   orc_greedy_coloring  TPZNumericalIntegrator.cpp:452-536
 *   orc_gather_strain    TPZNumericalIntegrator.cpp:40-51 + TPZIrregularBlocksMatrix.cpp:97-140 (opt 0)
 *   orc_scatter_residual TPZNumericalIntegrator.cpp:81-105 (alpha = -1, colour slabs,
 *                        pairwise slab reduction)
 *   orc_assemble_residual TPZElastoPlasticIntPointsStructMatrix.cpp:137-154
 *   orc_assemble         TPZElastoPlasticIntPointsStructMatrix.cpp:99-135 and
 *                        TPZNumericalIntegrator.cpp:131-182, 236-270 (element
 *                        tangent, upper triangle, colour-ordered accumulation)
 *   orc_solve_steps      main.cpp:160-262 (Newton) and main.cpp:487-522 (accept)
 * The mesh provider (quarter annulus, Q2 Lagrange basis, 3x3 Gauss, tractions,
 * Dirichlet symmetry) stands in for NeoPZ, which is not part of the reference.
 * Jacobi-PCG has no reference counterpart (the reference solves with Pardiso).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>
#include "orc_problem.h"

#define NB_NODES 256      /* nodes per level-1 reduction block */

/* ------------------------------------------------------------- utilities */

static void *xcalloc(size_t n, size_t s)
{
    void *p = calloc(n ? n : 1, s);
    if (!p) abort();
    return p;
}

static uint64_t sm64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}

static double urand(uint64_t seed, uint64_t e, uint64_t k)
{
    return (double)(sm64(seed * 0x100000001B3ULL + 4 * e + k) >> 11) * 0x1.0p-53;
}

void orc_default_params(orc_params *prm, int n)
{
    memset(prm, 0, sizeof *prm);
    prm->nr = n;
    prm->nt = n;
    prm->r_in = 0.1;
    prm->r_out = 4.0;
    prm->grading = pow(1.05, 40.0 / (double)n);
    prm->E = 15000.0;
    prm->nu = 0.2;
    prm->cohesion = 10.0;
    prm->phi_deg = 30.0;
    prm->psi_deg = 30.0;
    prm->sxx0 = -40.0;
    prm->syy0 = -50.0;
    prm->sxy0 = 0.0;
    prm->szz0 = 0.2 * (-40.0 + -50.0);
    prm->pw_final = -10.0;
    prm->material_mode = 0;
    prm->c_cv = 0.2;
    prm->phi_lo_deg = 25.0;
    prm->phi_hi_deg = 35.0;
    prm->seed = 20260101ULL;
}

/* -------------------------------------------------------- mesh provider */

void orc_vertex_coords(const orc_params *prm, double *vxy)
{
    const int nr = prm->nr, nt = prm->nt;
    const double q = prm->grading;
    double *r = (double *)xcalloc((size_t)nr + 1, sizeof(double));
    double h0 = (q == 1.0) ? (prm->r_out - prm->r_in) / (double)nr
                           : (prm->r_out - prm->r_in) * (q - 1.0) / (pow(q, (double)nr) - 1.0);
    r[0] = prm->r_in;
    for (int i = 0; i < nr - 1; i++) r[i + 1] = r[i] + h0 * pow(q, (double)i);
    r[nr] = prm->r_out;
    const double dth = (0.5 * M_PI) / (double)nt;
    for (int j = 0; j <= nt; j++) {
        double th = (double)j * dth;
        double c = cos(th), s = sin(th);
        for (int i = 0; i <= nr; i++) {
            double *v = &vxy[2 * ((size_t)j * (nr + 1) + i)];
            if (j == 0) { v[0] = r[i]; v[1] = 0.0; }
            else if (j == nt) { v[0] = 0.0; v[1] = r[i]; }
            else { v[0] = r[i] * c; v[1] = r[i] * s; }
        }
    }
    free(r);
}

/* reference coordinates of the 9 connects of order 2 (PZ quad order) */
static const int ref_a[9] = {-1, 1, 1, -1, 0, 1, 0, -1, 0};
static const int ref_b[9] = {-1, -1, 1, 1, -1, 0, 1, 0, 0};

static double lag(int a, double x)
{
    if (a < 0) return 0.5 * x * (x - 1.0);
    if (a == 0) return 1.0 - x * x;
    return 0.5 * x * (x + 1.0);
}

static double dlag(int a, double x)
{
    if (a < 0) return x - 0.5;
    if (a == 0) return -2.0 * x;
    return x + 0.5;
}

/* 1-D Lagrange function a of order p on the equispaced nodes t_m = -1 + 2m/p
 * and its derivative (orders 1 and 3; order 2 uses lag/dlag above) */
static double lagp(int p, int a, double x)
{
    const double ta = -1.0 + 2.0 * a / p;
    double num = 1.0, den = 1.0;
    for (int m = 0; m <= p; m++) {
        if (m == a) continue;
        const double tm = -1.0 + 2.0 * m / p;
        num = num * (x - tm);
        den = den * (ta - tm);
    }
    return num / den;
}

static double dlagp(int p, int a, double x)
{
    const double ta = -1.0 + 2.0 * a / p;
    double s = 0.0;
    for (int k = 0; k <= p; k++) {
        if (k == a) continue;
        const double tk = -1.0 + 2.0 * k / p;
        double prod = 1.0 / (ta - tk);
        for (int m = 0; m <= p; m++) {
            if (m == a || m == k) continue;
            const double tm = -1.0 + 2.0 * m / p;
            prod = prod * ((x - tm) / (ta - tm));
        }
        s = s + prod;
    }
    return s;
}

/* index-space position (a, b) in [0, p]^2 of connect n of an order-p element */
static void ref_node(int p, int n, int *a, int *b)
{
    const int vx[4] = {0, p, p, 0}, vy[4] = {0, 0, p, p};
    if (n < 4) { *a = vx[n]; *b = vy[n]; return; }
    n -= 4;
    if (n < 4 * (p - 1)) {
        const int e = n / (p - 1), k = n % (p - 1) + 1;
        if (e == 0) { *a = k; *b = 0; }
        else if (e == 1) { *a = p; *b = k; }
        else if (e == 2) { *a = p - k; *b = p; }
        else { *a = 0; *b = p - k; }
        return;
    }
    n -= 4 * (p - 1);
    *a = n % (p - 1) + 1;
    *b = n / (p - 1) + 1;
}

/* Gauss points and weights, p + 1 per direction */
static void gauss(int p, double *gp, double *gw)
{
    if (p == 1) {
        const double g = 1.0 / sqrt(3.0);
        gp[0] = -g; gp[1] = g;
        gw[0] = 1.0; gw[1] = 1.0;
    } else if (p == 2) {
        const double g = sqrt(0.6);
        gp[0] = -g; gp[1] = 0.0; gp[2] = g;
        gw[0] = 5.0 / 9.0; gw[1] = 8.0 / 9.0; gw[2] = 5.0 / 9.0;
    } else {
        const double a = sqrt(3.0 / 7.0 - 2.0 / 7.0 * sqrt(6.0 / 5.0));
        const double b = sqrt(3.0 / 7.0 + 2.0 / 7.0 * sqrt(6.0 / 5.0));
        const double wa = (18.0 + sqrt(30.0)) / 36.0, wb = (18.0 - sqrt(30.0)) / 36.0;
        gp[0] = -b; gp[1] = -a; gp[2] = a; gp[3] = b;
        gw[0] = wb; gw[1] = wa; gw[2] = wa; gw[3] = wb;
    }
}

void orc_element_blocks(int32_t order, int32_t n_el, const int32_t *connects, const double *node_xy,
                        double *B, double *weight)
{
    const int p = order, n1 = p + 1, nn = n1 * n1, nq = n1 * n1, nd = 2 * nn, nb = 3 * nq * nd;
    double gp[4], gw[4];
    gauss(p, gp, gw);
#pragma omp parallel for schedule(static)
    for (int32_t e = 0; e < n_el; e++) {
        double X[4], Y[4];
        for (int v = 0; v < 4; v++) {
            X[v] = node_xy[2 * (size_t)connects[(size_t)nn * e + v]];
            Y[v] = node_xy[2 * (size_t)connects[(size_t)nn * e + v] + 1];
        }
        double *Be = &B[(size_t)e * nb];
        memset(Be, 0, (size_t)nb * sizeof(double));
        for (int iq = 0; iq < nq; iq++) {
            const int ix = iq % n1, iy = iq / n1;
            const double xi = gp[ix], eta = gp[iy];
            const double dpx[4] = {-(1.0 - eta) / 4.0, (1.0 - eta) / 4.0, (1.0 + eta) / 4.0, -(1.0 + eta) / 4.0};
            const double dpe[4] = {-(1.0 - xi) / 4.0, -(1.0 + xi) / 4.0, (1.0 + xi) / 4.0, (1.0 - xi) / 4.0};
            double x_xi = dpx[0] * X[0], x_eta = dpe[0] * X[0];
            double y_xi = dpx[0] * Y[0], y_eta = dpe[0] * Y[0];
            for (int v = 1; v < 4; v++) {
                x_xi = x_xi + dpx[v] * X[v];
                x_eta = x_eta + dpe[v] * X[v];
                y_xi = y_xi + dpx[v] * Y[v];
                y_eta = y_eta + dpe[v] * Y[v];
            }
            const double det = x_xi * y_eta - x_eta * y_xi;
            const double xi_x = y_eta / det, xi_y = -x_eta / det;
            const double eta_x = -y_xi / det, eta_y = x_xi / det;
            weight[(size_t)e * nq + iq] = (gw[ix] * gw[iy]) * fabs(det);
            double *r0 = &Be[(3 * iq + 0) * nd];
            double *r1 = &Be[(3 * iq + 1) * nd];
            double *r2 = &Be[(3 * iq + 2) * nd];
            for (int n = 0; n < nn; n++) {
                double Nxi, Neta;
                if (p == 2) {
                    Nxi = dlag(ref_a[n], xi) * lag(ref_b[n], eta);
                    Neta = lag(ref_a[n], xi) * dlag(ref_b[n], eta);
                } else {
                    int a, b;
                    ref_node(p, n, &a, &b);
                    Nxi = dlagp(p, a, xi) * lagp(p, b, eta);
                    Neta = lagp(p, a, xi) * dlagp(p, b, eta);
                }
                const double dNx = Nxi * xi_x + Neta * eta_x;
                const double dNy = Nxi * xi_y + Neta * eta_y;
                r0[2 * n] = dNx;
                r1[2 * n] = dNy;
                r1[2 * n + 1] = dNx;
                r2[2 * n + 1] = dNy;
            }
        }
    }
}

int32_t orc_greedy_coloring_n(int32_t n_el, int32_t n_nodes, int32_t nn, const int32_t *connects,
                              int32_t *el_color)
{
    uint8_t *mark = (uint8_t *)xcalloc((size_t)n_nodes, 1);
    for (int32_t e = 0; e < n_el; e++) el_color[e] = -1;
    int32_t color = 0;
    int again = 1;
    while (again) {
        again = 0;
        for (int32_t e = 0; e < n_el; e++) {
            if (el_color[e] != -1) continue;
            const int32_t *c = &connects[(size_t)nn * e];
            int k;
            for (k = 0; k < nn; k++)
                if (mark[c[k]]) break;
            if (k != nn) { again = 1; continue; }
            el_color[e] = color;
            for (k = 0; k < nn; k++) mark[c[k]] = 1;
        }
        color++;
        memset(mark, 0, (size_t)n_nodes);
    }
    free(mark);
    return color;
}

int32_t orc_greedy_coloring(int32_t n_el, int32_t n_nodes, const int32_t *connects, int32_t *el_color)
{
    return orc_greedy_coloring_n(n_el, n_nodes, 9, connects, el_color);
}

static int cmp_i32(const void *a, const void *b)
{
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

/* edge traction of a uniform stress s = (sxx, sxy, syy) on segment P-M-Q,
 * outward normal sign sgn (+1: (dy,-dx)/L, -1: (-dy,dx)/L); Simpson weights */
static void seg_load(const double *xy, int32_t P, int32_t M, int32_t Q, int sgn,
                     double sxx, double sxy, double syy, double *f)
{
    const double dx = xy[2 * (size_t)Q] - xy[2 * (size_t)P];
    const double dy = xy[2 * (size_t)Q + 1] - xy[2 * (size_t)P + 1];
    const double L = sqrt(dx * dx + dy * dy);
    const double nx = sgn > 0 ? dy / L : -dy / L;
    const double ny = sgn > 0 ? -dx / L : dx / L;
    const double tx = sxx * nx + sxy * ny;
    const double ty = sxy * nx + syy * ny;
    const double we = L / 6.0, wm = 2.0 * L / 3.0;
    f[2 * (size_t)P] += tx * we;
    f[2 * (size_t)P + 1] += ty * we;
    f[2 * (size_t)M] += tx * wm;
    f[2 * (size_t)M + 1] += ty * wm;
    f[2 * (size_t)Q] += tx * we;
    f[2 * (size_t)Q + 1] += ty * we;
}

static void problem_setup(orc_problem *p, const orc_params *prm);

orc_problem *orc_problem_create(const orc_params *prm, int nthreads)
{
    if (nthreads > 0) omp_set_num_threads(nthreads);
    orc_problem *p = (orc_problem *)xcalloc(1, sizeof *p);
    p->prm = *prm;
    p->nthreads = nthreads > 0 ? nthreads : omp_get_max_threads();
    const int nr = prm->nr, nt = prm->nt;
    const int gr = 2 * nr + 1, gt = 2 * nt + 1;
    p->n_el = nr * nt;
    p->n_nodes = gr * gt;
    p->neq = 2 * p->n_nodes;
    p->order = 2;
    p->nn = p->nq = 9;
    p->nd = 18;
    p->n_ip = (int64_t)p->n_el * p->nq;

    /* nodes: vertex grid, then edge / centre nodes on the bilinear map */
    double *vxy = (double *)xcalloc((size_t)(nr + 1) * (nt + 1) * 2, sizeof(double));
    orc_vertex_coords(prm, vxy);
    p->node_xy = (double *)xcalloc((size_t)p->n_nodes * 2, sizeof(double));
    for (int b = 0; b < gt; b++)
        for (int a = 0; a < gr; a++) {
            double *o = &p->node_xy[2 * ((size_t)b * gr + a)];
            const int i0 = a / 2, j0 = b / 2;
            const int i1 = (a + 1) / 2, j1 = (b + 1) / 2;
            const double *v00 = &vxy[2 * ((size_t)j0 * (nr + 1) + i0)];
            const double *v10 = &vxy[2 * ((size_t)j0 * (nr + 1) + i1)];
            const double *v11 = &vxy[2 * ((size_t)j1 * (nr + 1) + i1)];
            const double *v01 = &vxy[2 * ((size_t)j1 * (nr + 1) + i0)];
            if (!(a & 1) && !(b & 1)) { o[0] = v00[0]; o[1] = v00[1]; }
            else if ((a & 1) && !(b & 1)) { o[0] = 0.5 * (v00[0] + v10[0]); o[1] = 0.5 * (v00[1] + v10[1]); }
            else if (!(a & 1) && (b & 1)) { o[0] = 0.5 * (v00[0] + v01[0]); o[1] = 0.5 * (v00[1] + v01[1]); }
            else {
                o[0] = 0.25 * (((v00[0] + v10[0]) + v11[0]) + v01[0]);
                o[1] = 0.25 * (((v00[1] + v10[1]) + v11[1]) + v01[1]);
            }
        }
    free(vxy);
    /* connects: element (i, j) = j*nr + i; vertices, edges, centre */
    p->connects = (int32_t *)xcalloc((size_t)p->n_el * 9, sizeof(int32_t));
    for (int j = 0; j < nt; j++)
        for (int i = 0; i < nr; i++) {
            int32_t *c = &p->connects[9 * ((size_t)j * nr + i)];
            const int a0 = 2 * i, b0 = 2 * j;
#define NID(a, b) ((int32_t)((b) * gr + (a)))
            c[0] = NID(a0, b0);         c[1] = NID(a0 + 2, b0);
            c[2] = NID(a0 + 2, b0 + 2); c[3] = NID(a0, b0 + 2);
            c[4] = NID(a0 + 1, b0);     c[5] = NID(a0 + 2, b0 + 1);
            c[6] = NID(a0 + 1, b0 + 2); c[7] = NID(a0, b0 + 1);
            c[8] = NID(a0 + 1, b0 + 1);
        }
    /* Dirichlet: u_y = 0 on y = 0 (b = 0), u_x = 0 on x = 0 (b = 2nt) */
    p->fixed = (uint8_t *)xcalloc((size_t)p->neq, 1);
    for (int a = 0; a < gr; a++) {
        p->fixed[2 * (size_t)NID(a, 0) + 1] = 1;
        p->fixed[2 * (size_t)NID(a, gt - 1) + 0] = 1;
    }
    /* loads: outer arc with sigma0, well arc with sigma0 -> pw I */
    p->f0 = (double *)xcalloc((size_t)p->neq, sizeof(double));
    p->df = (double *)xcalloc((size_t)p->neq, sizeof(double));
    {
        double *fo = (double *)xcalloc((size_t)p->neq, sizeof(double));
        double *fw0 = (double *)xcalloc((size_t)p->neq, sizeof(double));
        double *fw1 = (double *)xcalloc((size_t)p->neq, sizeof(double));
        for (int j = 0; j < nt; j++) {
            seg_load(p->node_xy, NID(gr - 1, 2 * j), NID(gr - 1, 2 * j + 1), NID(gr - 1, 2 * j + 2), +1,
                     prm->sxx0, prm->sxy0, prm->syy0, fo);
            seg_load(p->node_xy, NID(0, 2 * j), NID(0, 2 * j + 1), NID(0, 2 * j + 2), -1,
                     prm->sxx0, prm->sxy0, prm->syy0, fw0);
            seg_load(p->node_xy, NID(0, 2 * j), NID(0, 2 * j + 1), NID(0, 2 * j + 2), -1,
                     prm->pw_final, 0.0, prm->pw_final, fw1);
        }
        for (int32_t i = 0; i < p->neq; i++) {
            p->f0[i] = fo[i] + fw0[i];
            p->df[i] = fw1[i] - fw0[i];
        }
        free(fo); free(fw0); free(fw1);
    }
#undef NID
    problem_setup(p, prm);
    return p;
}

/* The same problem on a caller's quadrilateral mesh of order 1, 2 or 3
 * (connect order as in orc_problem.h; bilinear geometry from the vertices):
 * material, in-situ seed, setup and state as above. */
orc_problem *orc_problem_from_mesh(const orc_mesh_in *m, const orc_params *prm, int nthreads)
{
    if (nthreads > 0) omp_set_num_threads(nthreads);
    orc_problem *p = (orc_problem *)xcalloc(1, sizeof *p);
    p->prm = *prm;
    p->nthreads = nthreads > 0 ? nthreads : omp_get_max_threads();
    p->n_el = m->n_el;
    p->n_nodes = m->n_nodes;
    p->neq = 2 * m->n_nodes;
    p->order = m->order > 0 ? m->order : 2;
    p->nn = p->nq = (p->order + 1) * (p->order + 1);
    p->nd = 2 * p->nn;
    p->n_ip = (int64_t)p->n_el * p->nq;
    p->node_xy = (double *)xcalloc((size_t)p->n_nodes * 2, sizeof(double));
    memcpy(p->node_xy, m->node_xy, (size_t)p->n_nodes * 2 * sizeof(double));
    p->connects = (int32_t *)xcalloc((size_t)p->n_el * p->nn, sizeof(int32_t));
    memcpy(p->connects, m->connects, (size_t)p->n_el * p->nn * sizeof(int32_t));
    p->fixed = (uint8_t *)xcalloc((size_t)p->neq, 1);
    if (m->fixed) memcpy(p->fixed, m->fixed, (size_t)p->neq);
    p->f0 = (double *)xcalloc((size_t)p->neq, sizeof(double));
    p->df = (double *)xcalloc((size_t)p->neq, sizeof(double));
    if (m->f0) memcpy(p->f0, m->f0, (size_t)p->neq * sizeof(double));
    if (m->df) memcpy(p->df, m->df, (size_t)p->neq * sizeof(double));
    p->ext_dphi = m->dphi;
    p->ext_weight = m->weight;
    problem_setup(p, prm);
    p->ext_dphi = NULL;
    p->ext_weight = NULL;
    return p;
}

/* material, in-situ seed, B blocks, dof map, colouring, block pattern, state */
static void problem_setup(orc_problem *p, const orc_params *prm)
{
    /* material */
    orc_lame_from_engineering(prm->E, prm->nu, &p->el);
    p->mats = (orc_mc *)xcalloc((size_t)p->n_el, sizeof(orc_mc));
    {
        const double d2r = M_PI / 180.0;
        const double s2 = log(1.0 + prm->c_cv * prm->c_cv);
        const double mln = log(prm->cohesion) - 0.5 * s2;
        const double sln = sqrt(s2);
#pragma omp parallel for schedule(static)
        for (int32_t e = 0; e < p->n_el; e++) {
            double c = prm->cohesion, phi = prm->phi_deg, psi = prm->psi_deg;
            if (prm->material_mode >= 1) {
                double u1 = 1.0 - urand(prm->seed, (uint64_t)e, 0);
                double u2 = urand(prm->seed, (uint64_t)e, 1);
                double z = sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2);
                c = exp(mln + sln * z);
            }
            if (prm->material_mode >= 2) {
                phi = prm->phi_lo_deg + (prm->phi_hi_deg - prm->phi_lo_deg) * urand(prm->seed, (uint64_t)e, 2);
                psi = phi;
            }
            orc_mc_from_angles(c, phi * d2r, psi * d2r, &p->mats[e]);
        }
    }
    /* in-situ seed: eps_p0 = -C^{-1} sigma0, ComputeStrain (FunctionsStressStrain.h:73-81) */
    p->eps_p0 = (double *)xcalloc(6, sizeof(double));
    {
        const double lambda = p->el.lambda, mu = p->el.mu;
        const double s[6] = {prm->sxx0, prm->sxy0, 0.0, prm->syy0, 0.0, prm->szz0};
        double e6[6];
        e6[0] = (lambda + mu) / (3 * lambda * mu + 2 * mu * mu) * s[0] - lambda / (6 * lambda * mu + 4 * mu * mu) * (s[3] + s[5]);
        e6[3] = (lambda + mu) / (3 * lambda * mu + 2 * mu * mu) * s[3] - lambda / (6 * lambda * mu + 4 * mu * mu) * (s[0] + s[5]);
        e6[5] = (lambda + mu) / (3 * lambda * mu + 2 * mu * mu) * s[5] - lambda / (6 * lambda * mu + 4 * mu * mu) * (s[3] + s[0]);
        e6[1] = 1 / mu * s[1];
        e6[2] = 1 / mu * s[2];
        e6[4] = 1 / mu * s[4];
        for (int k = 0; k < 6; k++) p->eps_p0[k] = -e6[k];
    }
    /* setup: B blocks, weights, dof map, colouring */
    const int nn = p->nn, nd = p->nd;
    p->B = (double *)xcalloc((size_t)p->n_el * 3 * p->nq * nd, sizeof(double));
    p->weight = (double *)xcalloc((size_t)p->n_ip, sizeof(double));
    if (p->ext_dphi && p->ext_weight) {
        /* the caller's compact blocks into the fStorage layout */
        const int nq = p->nq, nb = 3 * nq * nd;
        for (int32_t e = 0; e < p->n_el; e++)
            for (int q = 0; q < nq; q++) {
                const double *dx = &p->ext_dphi[(((size_t)e * nq + q) * 2 + 0) * nn];
                const double *dy = &p->ext_dphi[(((size_t)e * nq + q) * 2 + 1) * nn];
                double *r0 = &p->B[(size_t)e * nb + (3 * q + 0) * nd];
                double *r1 = &p->B[(size_t)e * nb + (3 * q + 1) * nd];
                double *r2 = &p->B[(size_t)e * nb + (3 * q + 2) * nd];
                for (int n = 0; n < nn; n++) {
                    r0[2 * n] = dx[n];
                    r1[2 * n] = dy[n];
                    r1[2 * n + 1] = dx[n];
                    r2[2 * n + 1] = dy[n];
                }
            }
        memcpy(p->weight, p->ext_weight, (size_t)p->n_ip * sizeof(double));
    } else {
        orc_element_blocks(p->order, p->n_el, p->connects, p->node_xy, p->B, p->weight);
    }
    p->dofs = (int32_t *)xcalloc((size_t)p->n_el * nd, sizeof(int32_t));
    for (size_t k = 0; k < (size_t)p->n_el * nn; k++) {
        p->dofs[2 * k] = 2 * p->connects[k];
        p->dofs[2 * k + 1] = 2 * p->connects[k] + 1;
    }
    p->el_color = (int32_t *)xcalloc((size_t)p->n_el, sizeof(int32_t));
    p->n_colors = orc_greedy_coloring_n(p->n_el, p->n_nodes, nn, p->connects, p->el_color);
    p->color_ptr = (int32_t *)xcalloc((size_t)p->n_colors + 1, sizeof(int32_t));
    p->color_els = (int32_t *)xcalloc((size_t)p->n_el, sizeof(int32_t));
    for (int32_t e = 0; e < p->n_el; e++) p->color_ptr[p->el_color[e] + 1]++;
    for (int c = 0; c < p->n_colors; c++) p->color_ptr[c + 1] += p->color_ptr[c];
    {
        int32_t *fill = (int32_t *)xcalloc((size_t)p->n_colors, sizeof(int32_t));
        for (int32_t e = 0; e < p->n_el; e++) {
            int c = p->el_color[e];
            p->color_els[p->color_ptr[c] + fill[c]++] = e;
        }
        free(fill);
    }
    /* nodal block pattern: node -> sorted coupled nodes */
    {
        int32_t *deg = (int32_t *)xcalloc((size_t)p->n_nodes, sizeof(int32_t));
        int32_t *cnt = (int32_t *)xcalloc((size_t)p->n_nodes, sizeof(int32_t));
        for (int32_t e = 0; e < p->n_el; e++)
            for (int m = 0; m < nn; m++) cnt[p->connects[(size_t)nn * e + m]] += nn;
        int64_t *cap = (int64_t *)xcalloc((size_t)p->n_nodes + 1, sizeof(int64_t));
        for (int32_t i = 0; i < p->n_nodes; i++) cap[i + 1] = cap[i] + cnt[i];
        int32_t *tmp = (int32_t *)xcalloc((size_t)cap[p->n_nodes], sizeof(int32_t));
        for (int32_t e = 0; e < p->n_el; e++)
            for (int m = 0; m < nn; m++) {
                int32_t r = p->connects[(size_t)nn * e + m];
                for (int n = 0; n < nn; n++) tmp[cap[r] + deg[r]++] = p->connects[(size_t)nn * e + n];
            }
        p->row_ptr = (int64_t *)xcalloc((size_t)p->n_nodes + 1, sizeof(int64_t));
        for (int32_t i = 0; i < p->n_nodes; i++) {
            int32_t *s = &tmp[cap[i]];
            qsort(s, (size_t)deg[i], sizeof(int32_t), cmp_i32);
            int32_t u = 0;
            for (int32_t k = 0; k < deg[i]; k++)
                if (k == 0 || s[k] != s[k - 1]) s[u++] = s[k];
            deg[i] = u;
            p->row_ptr[i + 1] = p->row_ptr[i] + u;
        }
        p->n_blocks = p->row_ptr[p->n_nodes];
        p->col = (int32_t *)xcalloc((size_t)p->n_blocks, sizeof(int32_t));
        for (int32_t i = 0; i < p->n_nodes; i++)
            memcpy(&p->col[p->row_ptr[i]], &tmp[cap[i]], (size_t)deg[i] * sizeof(int32_t));
        free(tmp); free(cap); free(cnt); free(deg);
        p->el_blk = (int64_t *)xcalloc((size_t)p->n_el * nn * nn, sizeof(int64_t));
#pragma omp parallel for schedule(static)
        for (int32_t e = 0; e < p->n_el; e++)
            for (int m = 0; m < nn; m++) {
                int32_t r = p->connects[(size_t)nn * e + m];
                for (int n = 0; n < nn; n++) {
                    int32_t c = p->connects[(size_t)nn * e + n];
                    int64_t lo = p->row_ptr[r], hi = p->row_ptr[r + 1] - 1;
                    while (lo < hi) {
                        int64_t mid = (lo + hi) / 2;
                        if (p->col[mid] < c) lo = mid + 1; else hi = mid;
                    }
                    p->el_blk[((size_t)e * nn + m) * nn + n] = lo;
                }
            }
    }
    /* state */
    p->eps_p = (double *)xcalloc((size_t)p->n_ip * 6, sizeof(double));
    p->sigma = (double *)xcalloc((size_t)p->n_ip * 6, sizeof(double));
    p->mtype = (int8_t *)xcalloc((size_t)p->n_ip, 1);
    p->alpha = (double *)xcalloc((size_t)p->n_ip, sizeof(double));
    for (int64_t i = 0; i < p->n_ip; i++) {
        for (int k = 0; k < 6; k++) p->eps_p[6 * i + k] = p->eps_p0[k];
        p->sigma[6 * i + 0] = prm->sxx0;
        p->sigma[6 * i + 1] = prm->sxy0;
        p->sigma[6 * i + 3] = prm->syy0;
        p->sigma[6 * i + 5] = prm->szz0;
    }
    p->strain = (double *)xcalloc((size_t)p->n_ip * 3, sizeof(double));
    p->sigma_w = (double *)xcalloc((size_t)p->n_ip * 3, sizeof(double));
    p->dep = (double *)xcalloc((size_t)p->n_ip * 9, sizeof(double));
    p->K = (double *)xcalloc((size_t)p->n_blocks * 4, sizeof(double));
    p->dinv = (double *)xcalloc((size_t)p->neq, sizeof(double));
    p->binv = (double *)xcalloc((size_t)p->n_nodes * 4, sizeof(double));
}

void orc_problem_destroy(orc_problem *p)
{
    if (!p) return;
    free(p->binv);
    free(p->node_xy); free(p->connects); free(p->fixed); free(p->f0); free(p->df);
    free(p->mats); free(p->eps_p0); free(p->B); free(p->weight); free(p->dofs);
    free(p->el_color); free(p->color_ptr); free(p->color_els); free(p->row_ptr);
    free(p->col); free(p->el_blk); free(p->eps_p); free(p->sigma); free(p->mtype);
    free(p->alpha); free(p->strain); free(p->sigma_w); free(p->dep); free(p->K); free(p->dinv);
    free(p);
}

/* ------------------------------------------------------------ reductions */

static double tree32(double *v)
{
    for (int off = 16; off >= 1; off >>= 1)
        for (int l = 0; l < off; l++) v[l] = v[l] + v[l + off];
    return v[0];
}

int64_t orc_dot_partials(int64_t nnodes, const double *a, const double *b, double *partials)
{
    const int64_t nb = (nnodes + NB_NODES - 1) / NB_NODES;
#pragma omp parallel for schedule(static)
    for (int64_t blk = 0; blk < nb; blk++) {
        double w[8];
        for (int s = 0; s < 8; s++) {
            double v[32];
            for (int l = 0; l < 32; l++) {
                int64_t n = blk * NB_NODES + 32 * s + l;
                double acc = 0.0;
                if (n < nnodes) {
                    acc = fma(a[2 * n], b[2 * n], acc);
                    acc = fma(a[2 * n + 1], b[2 * n + 1], acc);
                }
                v[l] = acc;
            }
            w[s] = tree32(v);
        }
        for (int off = 4; off >= 1; off >>= 1)
            for (int l = 0; l < off; l++) w[l] = w[l] + w[l + off];
        partials[blk] = w[0];
    }
    return nb;
}

double orc_dot_final(int64_t np, const double *partials)
{
    double acc[256];
    for (int t = 0; t < 256; t++) {
        double s = 0.0;
        for (int64_t k = t; k < np; k += 256) s = s + partials[k];
        acc[t] = s;
    }
    double ws[8];
    for (int w = 0; w < 8; w++) ws[w] = tree32(&acc[32 * w]);
    for (int off = 4; off >= 1; off >>= 1)
        for (int l = 0; l < off; l++) ws[l] = ws[l] + ws[l + off];
    return ws[0];
}

double orc_dot(int64_t nnodes, const double *a, const double *b)
{
    const int64_t nb = (nnodes + NB_NODES - 1) / NB_NODES;
    double *part = (double *)xcalloc((size_t)nb, sizeof(double));
    orc_dot_partials(nnodes, a, b, part);
    double r = orc_dot_final(nb, part);
    free(part);
    return r;
}

/* ------------------------------------------------------------- assembly */

void orc_gather_strain(const orc_problem *p, const double *u, double *strain)
{
#pragma omp parallel for schedule(static)
    for (int32_t e = 0; e < p->n_el; e++) {
        const int nd = p->nd, nr = 3 * p->nq;
        double ue[32];
        for (int j = 0; j < nd; j++) ue[j] = u[p->dofs[(size_t)nd * e + j]];
        const double *Be = &p->B[(size_t)e * nr * nd];
        for (int r = 0; r < nr; r++) {
            double acc = 0.0;
            for (int j = 0; j < nd; j++) acc = fma(Be[r * nd + j], ue[j], acc);
            strain[(size_t)e * nr + r] = acc;
        }
    }
}

void orc_scatter_residual(const orc_problem *p, const double *sigma_w, double *res)
{
    const int32_t neq = p->neq;
    const int nc = p->n_colors;
    double *slab = (double *)xcalloc((size_t)nc * neq, sizeof(double));
#pragma omp parallel for schedule(static)
    for (int32_t e = 0; e < p->n_el; e++) {
        const int nd = p->nd, nr = 3 * p->nq;
        const double *Be = &p->B[(size_t)e * nr * nd];
        const double *s = &sigma_w[(size_t)e * nr];
        double *sl = &slab[(size_t)p->el_color[e] * neq];
        for (int j = 0; j < nd; j++) {
            double acc = 0.0;
            for (int r = 0; r < nr; r++) acc = fma(Be[r * nd + j], s[r], acc);
            sl[p->dofs[(size_t)nd * e + j]] = -acc;
        }
    }
    int64_t ncol = nc, ca = nc / 2;
    while (ca > 0) {
        const int64_t first = (ncol - ca) * (int64_t)neq;
        const int64_t len = ca * (int64_t)neq;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < len; i++) slab[i] = slab[i] + slab[first + i];
        ncol -= ca;
        ca = ncol / 2;
    }
    memcpy(res, slab, (size_t)neq * sizeof(double));
    free(slab);
}

static void finish_rhs(const orc_problem *p, double lambda, double *rhs)
{
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < p->neq; i++) {
        const double lin = fma(lambda, p->df[i], p->f0[i]);
        rhs[i] = p->fixed[i] ? 0.0 : rhs[i] + lin;
    }
}

void orc_assemble_residual(orc_problem *p, const double *u, double lambda, int update_mem, double *rhs)
{
    orc_gather_strain(p, u, p->strain);
    orc_compute_sigma_batch(p->n_ip, p->nq, &p->el, p->mats, p->strain, p->eps_p, p->weight,
                            update_mem, p->sigma_w, 0, p->sigma, p->mtype, p->alpha);
    orc_scatter_residual(p, p->sigma_w, rhs);
    finish_rhs(p, lambda, rhs);
}

void orc_assemble(orc_problem *p, const double *u, double lambda, double *rhs)
{
    orc_gather_strain(p, u, p->strain);
    orc_compute_sigma_batch(p->n_ip, p->nq, &p->el, p->mats, p->strain, p->eps_p, p->weight,
                            0, p->sigma_w, p->dep, 0, 0, 0);
    orc_scatter_residual(p, p->sigma_w, rhs);
    finish_rhs(p, lambda, rhs);
    memset(p->K, 0, (size_t)p->n_blocks * 4 * sizeof(double));
    for (int c = 0; c < p->n_colors; c++) {
#pragma omp parallel for schedule(static)
        for (int32_t k = p->color_ptr[c]; k < p->color_ptr[c + 1]; k++) {
            const int32_t e = p->color_els[k];
            const int nn = p->nn, nq = p->nq, nd = p->nd;
            const double *Be = &p->B[(size_t)e * 3 * nq * nd];
            double Kl[32][32];
            memset(Kl, 0, sizeof Kl);
            for (int q = 0; q < nq; q++) {
                const double *Bq = &Be[q * 3 * nd];
                const double *D = &p->dep[((size_t)e * nq + q) * 9];
                double DB[3][32];
                for (int i = 0; i < 3; i++)
                    for (int j = 0; j < nd; j++) {
                        double s = D[3 * i + 0] * Bq[0 * nd + j];
                        s = fma(D[3 * i + 1], Bq[1 * nd + j], s);
                        s = fma(D[3 * i + 2], Bq[2 * nd + j], s);
                        DB[i][j] = s;
                    }
                for (int a = 0; a < nd; a++)
                    for (int b = a; b < nd; b++) {
                        double t = Kl[a][b];
                        t = fma(Bq[0 * nd + a], DB[0][b], t);
                        t = fma(Bq[1 * nd + a], DB[1][b], t);
                        t = fma(Bq[2 * nd + a], DB[2][b], t);
                        Kl[a][b] = t;
                    }
            }
            const int64_t *eb = &p->el_blk[(size_t)e * nn * nn];
            for (int a = 0; a < nd; a++)
                for (int b = a; b < nd; b++) {
                    const int m = a / 2, ca = a % 2, n = b / 2, cb = b % 2;
                    const double v = Kl[a][b];
                    if (m == n) {
                        double *blk = &p->K[4 * eb[m * nn + m]];
                        blk[2 * ca + cb] = blk[2 * ca + cb] + v;
                        if (ca != cb) blk[2 * cb + ca] = blk[2 * cb + ca] + v;
                    } else {
                        double *b1 = &p->K[4 * eb[m * nn + n]];
                        double *b2 = &p->K[4 * eb[n * nn + m]];
                        b1[2 * ca + cb] = b1[2 * ca + cb] + v;
                        b2[2 * cb + ca] = b2[2 * cb + ca] + v;
                    }
                }
        }
    }
    /* Jacobi: inverse of the nodal-block diagonal entries on free dofs */
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < p->n_nodes; i++) {
        int64_t lo = p->row_ptr[i], hi = p->row_ptr[i + 1] - 1;
        while (lo < hi) {
            int64_t mid = (lo + hi) / 2;
            if (p->col[mid] < i) lo = mid + 1; else hi = mid;
        }
        const double *blk = &p->K[4 * lo];
        p->dinv[2 * i] = p->fixed[2 * i] ? 0.0 : 1.0 / blk[0];
        p->dinv[2 * i + 1] = p->fixed[2 * i + 1] ? 0.0 : 1.0 / blk[3];
        /* block Jacobi: the inverse of the 2x2 diagonal block on the free dofs */
        const int fx = p->fixed[2 * i], fy = p->fixed[2 * i + 1];
        double *m = &p->binv[4 * (size_t)i];
        m[0] = m[1] = m[2] = m[3] = 0.0;
        if (!fx && !fy) {
            const double det = blk[0] * blk[3] - blk[1] * blk[2];
            m[0] = blk[3] / det;
            m[1] = -blk[1] / det;
            m[2] = -blk[2] / det;
            m[3] = blk[0] / det;
        } else if (!fx) {
            m[0] = 1.0 / blk[0];
        } else if (!fy) {
            m[3] = 1.0 / blk[3];
        }
    }
}

void orc_spmv(const orc_problem *p, const double *x, double *y)
{
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < p->n_nodes; i++) {
        double y0 = 0.0, y1 = 0.0;
        for (int64_t k = p->row_ptr[i]; k < p->row_ptr[i + 1]; k++) {
            const double *a = &p->K[4 * k];
            const double x0 = x[2 * (size_t)p->col[k]], x1 = x[2 * (size_t)p->col[k] + 1];
            y0 = fma(a[0], x0, y0);
            y0 = fma(a[1], x1, y0);
            y1 = fma(a[2], x0, y1);
            y1 = fma(a[3], x1, y1);
        }
        y[2 * (size_t)i] = p->fixed[2 * i] ? 0.0 : y0;
        y[2 * (size_t)i + 1] = p->fixed[2 * i + 1] ? 0.0 : y1;
    }
}

/* z = M r: Jacobi (z_i = r_i / K_ii on free dofs) or block Jacobi
 * (z = B_i^-1 r at node i, z0 = fma(m01, r1, m00 r0), z1 = fma(m11, r1, m10 r0)) */
static void precondition(const orc_problem *p, const double *r, double *z)
{
    if (p->cg_block) {
#pragma omp parallel for schedule(static)
        for (int32_t i = 0; i < p->n_nodes; i++) {
            const double *m = &p->binv[4 * (size_t)i];
            const double r0 = r[2 * i], r1 = r[2 * i + 1];
            z[2 * i] = fma(m[1], r1, m[0] * r0);
            z[2 * i + 1] = fma(m[3], r1, m[2] * r0);
        }
    } else {
#pragma omp parallel for schedule(static)
        for (int32_t i = 0; i < p->neq; i++) z[i] = r[i] * p->dinv[i];
    }
}

int orc_pcg(const orc_problem *p, const double *b, double *x, double rtol, int max_it, double *work)
{
    const int32_t n = p->neq;
    const int64_t nn = p->n_nodes;
    double *r = work, *z = work + n, *pv = work + 2 * (size_t)n, *q = work + 3 * (size_t)n;
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < n; i++) {
        x[i] = 0.0;
        r[i] = b[i];
    }
    precondition(p, r, z);
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < n; i++) pv[i] = z[i];
    const double bb = orc_dot(nn, b, b);
    if (bb == 0.0) return 0;
    const double thr = (rtol * rtol) * bb;
    double rz = orc_dot(nn, r, z);
    for (int k = 1; k <= max_it; k++) {
        orc_spmv(p, pv, q);
        const double pq = orc_dot(nn, pv, q);
        if (!(pq > 0.0)) return -k;
        const double alpha = rz / pq;
#pragma omp parallel for schedule(static)
        for (int32_t i = 0; i < n; i++) {
            x[i] = fma(alpha, pv[i], x[i]);
            r[i] = fma(-alpha, q[i], r[i]);
        }
        precondition(p, r, z);
        const double rr = orc_dot(nn, r, r);
        if (rr <= thr) return k;
        const double rzn = orc_dot(nn, r, z);
        const double beta = rzn / rz;
        rz = rzn;
#pragma omp parallel for schedule(static)
        for (int32_t i = 0; i < n; i++) pv[i] = fma(beta, pv[i], z[i]);
    }
    return -max_it;
}

void orc_solve_steps(orc_problem *p, const orc_solve_opts *o, int32_t step_begin, int32_t step_end,
                     double *u, orc_solve_stats *st, double *log, int32_t log_cap)
{
    const int32_t n = p->neq;
    double *R = (double *)xcalloc((size_t)n, sizeof(double));
    double *du = (double *)xcalloc((size_t)n, sizeof(double));
    double *work = (double *)xcalloc((size_t)n * 4, sizeof(double));
    double *t = o->accel ? (double *)xcalloc((size_t)n, sizeof(double)) : NULL;
    int32_t nlog = 0;
    int have_k = 0;
    memset(st, 0, sizeof *st);
    st->converged = 1;
    /* tangent_mode 1, the initial-stiffness iteration of the reference's
     * logged runs (the initial-stiffness branch of Solution(), main.cpp:218-222, with only the residual
     * assembled per iteration): K and the Jacobi diagonal of the first
     * assembly are kept, later assemblies compute the residual alone */
#define ASSEMBLE_ITER()                                          \
    do {                                                         \
        if (o->tangent_mode == 1 && have_k) {                    \
            orc_assemble_residual(p, u, lambda, 0, R);           \
        } else {                                                 \
            orc_assemble(p, u, lambda, R);                       \
            have_k = 1;                                          \
        }                                                        \
    } while (0)
    for (int32_t s = step_begin; s < step_end; s++) {
        const double lambda = (double)(s + 1) / (double)o->n_steps;
        ASSEMBLE_ITER();
        const double r0 = sqrt(orc_dot(p->n_nodes, R, R));
        double rn = r0;
        int conv = (r0 == 0.0);
        int it = 0;
        double alpha = 1.0;                          /* main.cpp:170, reset per load step */
        while (!conv && it < o->newton_max_it) {
            int k = orc_pcg(p, R, du, o->cg_rtol, o->cg_max_it, work);
            st->cg_iters += k < 0 ? -k : k;
            if (o->accel) {
                /* main.cpp:194-217: u += alpha du, residual at u, second solve
                 * with the same tangent, alpha += (alpha du . du~) / |alpha du|^2,
                 * u += du~ (alpha unchanged when alpha du = 0) */
                for (int32_t i = 0; i < n; i++) {
                    t[i] = alpha * du[i];
                    u[i] = u[i] + t[i];
                }
                orc_assemble_residual(p, u, lambda, 0, R);
                int k2 = orc_pcg(p, R, du, o->cg_rtol, o->cg_max_it, work);
                st->cg_iters += k2 < 0 ? -k2 : k2;
                k = (k < 0 ? -k : k) + (k2 < 0 ? -k2 : k2);
                const double num = orc_dot(p->n_nodes, t, du), dem = orc_dot(p->n_nodes, t, t);
                if (dem > 0.0) alpha = alpha + num / dem;
            }
            for (int32_t i = 0; i < n; i++) u[i] = u[i] + du[i];
            it++;
            ASSEMBLE_ITER();
            rn = sqrt(orc_dot(p->n_nodes, R, R));
            if (log && nlog < log_cap) {
                log[3 * nlog + 0] = (double)s;
                log[3 * nlog + 1] = (double)k;
                log[3 * nlog + 2] = rn;
                nlog++;
            }
            conv = rn <= o->newton_rtol * r0;
        }
        st->newton_iters += it;
        st->last_step_iters = it;
        st->final_res = r0 > 0.0 ? rn / r0 : 0.0;
        if (!conv) st->converged = 0;
        orc_assemble_residual(p, u, lambda, 1, R);     /* accept: commit state */
    }
    free(R); free(du); free(work); free(t);
#undef ASSEMBLE_ITER
}
