/*
 * CPU oracle (test infrastructure only): the wellbore problem, its setup and
 * the assembly / solve steps of the reference path, restated in C.
 * See ipfem_oracle.h for the arithmetic conventions.
 */
#ifndef IPFEM_ORC_PROBLEM_H
#define IPFEM_ORC_PROBLEM_H

#include <stdint.h>
#include "ipfem_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Element order p (1, 2, 3): (p+1)^2 connects and (p+1)^2 Gauss points per
 * quadrilateral, 2 (p+1)^2 dofs; the wellbore provider builds order 2.
 * Connect order of an element: 4 vertices, the p-1 nodes of each edge in the
 * element's traversal direction (edges v0v1, v1v2, v2v3, v3v0), interior
 * nodes row by row. */
#define ORC_NPTS 9      /* order 2: 3x3 Gauss points */
#define ORC_NNODE 9     /* order 2: connects per element */
#define ORC_NDOF 18     /* order 2: element dofs */

typedef struct {
    int32_t nr, nt;            /* elements in radial / angular direction */
    double r_in, r_out;        /* radii */
    double grading;            /* radial size ratio between neighbouring cells */
    double E, nu;
    double cohesion, phi_deg, psi_deg;
    double sxx0, syy0, sxy0, szz0;  /* in-situ stress (compression negative) */
    double pw_final;           /* well-wall sigma_rr at lambda = 1 (signed) */
    int32_t material_mode;     /* 0 uniform; 1 lognormal cohesion; 2 + uniform phi=psi */
    double c_cv;               /* coefficient of variation of cohesion */
    double phi_lo_deg, phi_hi_deg;
    uint64_t seed;
} orc_params;

typedef struct {
    orc_params prm;
    int32_t n_el, n_nodes, neq;
    int64_t n_ip;
    /* mesh provider (stand-in for the NeoPZ geometric/computational mesh) */
    double *node_xy;           /* [n_nodes*2] */
    int32_t *connects;         /* [n_el*nn] connect order: vertices, edge nodes, interior */
    uint8_t *fixed;            /* [neq] strong Dirichlet dofs */
    double *f0, *df;           /* [neq] external load = f0 + lambda*df */
    orc_elastic el;
    orc_mc *mats;              /* [n_el] */
    double *eps_p0;            /* [6] in-situ plastic-strain seed -C^{-1} sigma0 */
    /* setup (TPZNumericalIntegrator::SetUp*) */
    double *B;                 /* [n_el*(3 nq)*nd] row-major element blocks (fStorage) */
    double *weight;            /* [n_ip] */
    int32_t *dofs;             /* [n_el*nd] fDoFIndexes */
    int32_t n_colors;
    int32_t *el_color;         /* [n_el] */
    int32_t *color_ptr;        /* [n_colors+1] */
    int32_t *color_els;        /* [n_el] fElColorIndex */
    /* nodal 2x2 block sparsity (full, both triangles) */
    int64_t n_blocks;
    int64_t *row_ptr;          /* [n_nodes+1] */
    int32_t *col;              /* [n_blocks] ascending per row */
    int64_t *el_blk;           /* [n_el*nn*nn] block index of local node pair (m,n) */
    /* state at integration points (committed) */
    double *eps_p;             /* [n_ip*6] */
    double *sigma;             /* [n_ip*6] */
    int8_t *mtype;             /* [n_ip] */
    double *alpha;             /* [n_ip] */
    /* work */
    double *strain;            /* [n_ip*3] */
    double *sigma_w;           /* [n_ip*3] */
    double *dep;               /* [n_ip*9] */
    double *K;                 /* [n_blocks*4] */
    double *dinv;              /* [neq] */
    int nthreads;
    int32_t order, nn, nq, nd; /* element order; connects, points, dofs per element */
    double *binv;              /* [n_nodes*4] inverse of each nodal diagonal block on its free dofs */
    int32_t cg_block;          /* 1: orc_pcg preconditions with binv (block Jacobi), 0: dinv */
    const double *ext_dphi, *ext_weight;   /* caller's element blocks during construction only */
} orc_problem;

orc_problem *orc_problem_create(const orc_params *prm, int nthreads);
/* a caller's order-2 mesh; prm supplies the material and in-situ stress
 * (its mesh fields are ignored) */
typedef struct {
    int32_t n_el, n_nodes;
    const double *node_xy;     /* [n_nodes*2] */
    const int32_t *connects;   /* [n_el*9] */
    const uint8_t *fixed;      /* [2*n_nodes] or NULL */
    const double *f0, *df;     /* [2*n_nodes] or NULL */
    int32_t order;             /* 1, 2 or 3 (0 = 2) */
    /* element blocks given by the caller (elements that are not bilinear
     * quadrilaterals, e.g. padded triangles), or NULL: computed from node_xy */
    const double *dphi;        /* [n_el*nq*2*nn] d(phi_n)/d(x_d) at point q, ((e*nq+q)*2+d)*nn+n */
    const double *weight;      /* [n_el*nq] */
} orc_mesh_in;
orc_problem *orc_problem_from_mesh(const orc_mesh_in *m, const orc_params *prm, int nthreads);
void orc_problem_destroy(orc_problem *p);
void orc_default_params(orc_params *prm, int n);

/* setup pieces (exposed for tests) */
void orc_vertex_coords(const orc_params *prm, double *vxy);
void orc_element_blocks(int32_t order, int32_t n_el, const int32_t *connects, const double *node_xy,
                        double *B, double *weight);
int32_t orc_greedy_coloring(int32_t n_el, int32_t n_nodes, const int32_t *connects, int32_t *el_color);

/* TPZNumericalIntegrator::Multiply: strain = B * u[dofs] */
void orc_gather_strain(const orc_problem *p, const double *u, double *strain);
/* TPZNumericalIntegrator::MultiplyTranspose: res = colored-reduced (-B^T sigma_w) */
void orc_scatter_residual(const orc_problem *p, const double *sigma_w, double *res);
/* Assemble(rhs): rhs = -B^T sigma(u) + f(lambda), Dirichlet rows zeroed */
void orc_assemble_residual(orc_problem *p, const double *u, double lambda, int update_mem, double *rhs);
/* Assemble(K, rhs): also the tangent into p->K and the Jacobi inverse diagonal */
void orc_assemble(orc_problem *p, const double *u, double lambda, double *rhs);
/* y = K x on free dofs, 0 on fixed dofs */
void orc_spmv(const orc_problem *p, const double *x, double *y);
/* Jacobi-PCG: K x = b.  x is overwritten (starts from 0).  Returns iterations
 * (negative if max_it reached). */
int orc_pcg(const orc_problem *p, const double *b, double *x, double rtol, int max_it,
            double *work /* 4*neq */);

typedef struct {
    int32_t n_steps;
    double newton_rtol;
    int32_t newton_max_it;
    double cg_rtol;
    int32_t cg_max_it;
    int32_t accel;             /* 1: modified-Thomas acceleration (main.cpp:194-217) */
    int32_t tangent_mode;      /* 1: initial stiffness (K of the first assembly kept) */
} orc_solve_opts;

typedef struct {
    int32_t newton_iters;      /* total over the steps run */
    int64_t cg_iters;
    int32_t last_step_iters;
    int32_t converged;         /* all steps converged */
    double final_res;          /* |R| / |R0| of the last step */
} orc_solve_stats;

/* Load-stepped Newton (main.cpp:160-262 per step, accept = main.cpp:487-522).
 * Runs steps [step_begin, step_end) of n_steps, u is updated in place;
 * per-iteration log (newton_it, cg_its, |R|) written into log if not NULL
 * (log_cap entries of 3 doubles). */
void orc_solve_steps(orc_problem *p, const orc_solve_opts *o, int32_t step_begin, int32_t step_end,
                     double *u, orc_solve_stats *st, double *log, int32_t log_cap);

#ifdef __cplusplus
}
#endif

#endif
