/*
 * CPU oracle for the integration-point residual / Newton-CG path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (libipfem.so and the
 * intpointsfem_gb300 package) links, loads or calls this code.  It is used by
 * tests/ (as the parity checker), by __graft_entry__.smoke() (as the checker)
 * and by bench.py's CPU-baseline leg (as the timed CPU restatement).
 *
 * It restates, in plain C, the algorithm of labmec/IntPointsFEM for this
 * path.  Every function cites the reference file:line it follows.  The
 * constitutive part (Functions*.h) is checked bit-for-bit against the
 * reference's own headers compiled under oracle/_ref (see oracle/build.py and
 * tests/golden/make_golden.py).
 *
 * Arithmetic conventions (shared with the CUDA product so results can be
 * compared bit-for-bit):
 *   - constitutive update: plain IEEE mul/add/div/sqrt in the reference's
 *     operation order, no contraction (-ffp-contract=off), trigonometric
 *     values of phi/psi computed once per material by libm;
 *   - block products (B*u, B^T*sigma, element stiffness, SpMV, dots, axpys):
 *     explicit fma() in a fixed, documented order;
 *   - reductions: the canonical two-level tree of orc_dot().
 */
#ifndef IPFEM_ORACLE_H
#define IPFEM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- material */
/* Per-element Mohr-Coulomb constants.  Trigonometry is evaluated once by the
 * host (libm) and shared by oracle and device code. */
typedef struct {
    double cohesion;
    double sinphi, cosphi, tanphi;   /* friction angle phi */
    double sinpsi;                   /* dilation angle psi */
} orc_mc;

/* Elastic constants (uniform over the mesh). */
typedef struct {
    double lambda, mu;               /* Lame constants */
} orc_elastic;

void orc_mc_from_angles(double cohesion, double phi, double psi, orc_mc *out);
void orc_lame_from_engineering(double E, double nu, orc_elastic *out);

/* One integration point, CPU-path sequence of
 * TPZConstitutiveLawProcessor::ComputeSigma (TPZConstitutiveLawProcessor.cpp:150-211)
 * and ::ComputeSigmaDep (…cpp:364-439).
 *   strain3    : B*u at the point, (eps_xx, gamma_xy, eps_yy)
 *   eps_p6     : committed plastic strain, 6 comps {XX,XY,XZ,YY,YZ,ZZ}
 *   weight     : w*|detJ|
 * outputs:
 *   sigma_w3   : weight*(s_xx, s_xy, s_yy)
 *   dep9       : weight*Dep (3x3 row-major, XY column halved), NULL = no tangent
 *   sigma6     : stress 6 comps
 *   eps_p6_out : updated plastic strain 6 comps
 *   strain6    : composed total strain 6 comps
 *   mtype      : 0 elastic, 1 plane/edge, -1 apex
 *   alpha      : hardening increment accumulated from 0
 */
void orc_ip_update(const orc_elastic *el, const orc_mc *mc,
                   const double strain3[3], const double eps_p6[6], double weight,
                   double sigma_w3[3], double *dep9,
                   double sigma6[6], double eps_p6_out[6], double strain6[6],
                   int *mtype, double *alpha);

/* Tangent variant for Newton studies: 0 (default) the reference's
 * TangentOperator; 1 the consistent spectral tangent (spin factors from the
 * projected principal stresses, one ProdT pair per eigen-pair).  Global. */
void orc_set_consistent_tangent(int on);

/* Point update with the full 6x6 tangent (XX XY XZ YY YZ ZZ; row = stress,
 * column = strain), as TPZPlasticStepPV::ApplyStrainComputeSigma's Dep that
 * TRKSolution::RKProcess reads (TRKSolution.cpp:189-191). */
/* Decomposition variant for studies: 0 (default) the reference's
 * SpectralDecomposition; 1 the closed form of plane-strain tensors (XZ = YZ
 * = 0): ZZ and the in-plane 2x2 eigen-pairs.  Global. */
void orc_set_spectral_mode(int mode);

/* SpectralDecomposition (FunctionsSpectralDecomp.h:261-268) of one symmetric
 * tensor: eigenvalues in descending order, eigenvectors as rows of vec9. */
void orc_spectral(const double s6[6], double ev[3], double vec9[9]);

void orc_ip_tangent6(const orc_elastic *el, const orc_mc *mc, const double strain6[6], const double eps_p6[6],
                     double sigma6[6], double eps_p6_out[6], double T36[36], int *mtype);

/* Same, but with the argument aliasing of the reference GPU residual kernel
 * (KernelsComputeSigma.h:48: ProjectSigma(sigma_projected, sigma_projected, ...)).
 * Only used to document the CPU/GPU discrepancy of the reference. */
void orc_ip_update_gpu_alias(const orc_elastic *el, const orc_mc *mc,
                             const double strain3[3], const double eps_p6[6], double weight,
                             double sigma_w3[3], double sigma6[6], double eps_p6_out[6],
                             int *mtype, double *alpha);

/* Batched constitutive update over npts points.  Point i uses material
 * mats[i / pts_per_mat].  State arrays are AoS with the reference strides
 * (3 for strain/sigma_w, 6 for plastic strain, 9 for dep).  dep may be NULL.
 * If update_mem != 0, eps_p6 is overwritten with the updated plastic strain
 * and sigma6_state / mtype / alpha receive the committed values (the GPU
 * assignment semantics of KernelsComputeSigma.h:59-68). */
void orc_compute_sigma_batch(int64_t npts, int pts_per_mat,
                             const orc_elastic *el, const orc_mc *mats,
                             const double *strain3, double *eps_p6,
                             const double *weight, int update_mem,
                             double *sigma_w3, double *dep9,
                             double *sigma6_state, int8_t *mtype, double *alpha);

/* ---------------------------------------------------------------- reductions */
/* Canonical deterministic dot product over n2 = 2*nnodes doubles laid out as
 * node-interleaved pairs.  Level 0: lane l of a 32-lane slice handles node
 * 32*s+l: acc = fma(a[2n],b[2n],0); acc = fma(a[2n+1],b[2n+1],acc); the 32
 * lanes are folded by the shuffle-down tree (16,8,4,2,1).  Level 1: the 8
 * slice sums of a 256-node block are folded by the tree (4,2,1).  Level 2:
 * the block partials are strided over 256 threads (t, t+256, ... summed in
 * order from 0), each warp folds by (16..1), and the 8 warp sums by (4,2,1). */
double orc_dot(int64_t nnodes, const double *a, const double *b);
/* the three levels separately (exposed for tests) */
int64_t orc_dot_partials(int64_t nnodes, const double *a, const double *b, double *partials);
double orc_dot_final(int64_t npartials, const double *partials);

#ifdef __cplusplus
}
#endif

#endif
