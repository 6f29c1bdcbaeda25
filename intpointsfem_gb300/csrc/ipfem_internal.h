// Internal declarations shared by the host setup (C++) and the CUDA
// translation units of libipfem.  Not part of the C-ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <string>
#include <vector>

#include "../../include/ipfem.h"

namespace ipfem {

constexpr int kMaxColors = 16;
constexpr int kRedBlock = 256;       // nodes per level-1 reduction block (= CTA size)
constexpr int kPatLen = 32;          // offsets per row stencil (longest row that can use one)
constexpr int kPatMax = 255;         // row stencils per layout (ids are 8-bit)

struct ElasticConstH {               // mirrors ElasticConst of constitutive.cuh
    double lambda, mu, K, G, l2m, c1, c2, inv_mu;
};

// device-side scalars of one CG solve
template <class T>
struct CGScalarsT {
    T rz, pq, alpha, beta, rr, bb, thr;
    int done, iters, status, max_it;
    T rr_best;                    // flexible CG: stagnation watch
    int it_best, fallback;
};
constexpr int kStatusFallback = 9;   // flexible CG stagnated: the caller falls back to Jacobi-PCG
// codes of the device error word (bounded waits that gave up)
constexpr int kErrBulkWait = 1;      // a bulk (TMA) copy did not complete (3: a tensor-core pipeline wait)
typedef CGScalarsT<double> CGScalars;

// SELL-32 layout of the nodal 2x2 block pattern: row position t of slice
// t/32 holds node sell_node[t] (identity when the rows keep node order).
// Its block k sits in slot slice_base[t/32] + 32*k + t%32, or, with slot
// pairs, in slot slice_base[t/32] + 64*(k/2) + 2*(t%32) + k%2: two blocks of
// one row side by side, so that a 32-byte sector of FP32 blocks never holds
// a block of a shorter neighbouring row's padding (slices are then padded to
// an even width).
struct SellLayout {
    bool pair = false;                   // slot pairs (the FP32 layout)
    int64_t n_sell = 0;                  // padded block slots
    std::vector<int64_t> slice_base;     // [n_slices+1], in blocks
    std::vector<int32_t> sell_node;      // [n_nodes] node at each row position
    std::vector<int32_t> rowlen;         // [n_nodes] blocks of the row at each row position
    std::vector<int32_t> sell_col;       // [n_sell]
    std::vector<int64_t> bsr_to_sell;    // [n_blocks]
    std::vector<int32_t> el_blk;         // [n_el*nn*nn] slot of local node pair (m, n)
    std::vector<int64_t> diag_blk;       // [n_nodes] slot of the diagonal block
    // row stencils (build_row_stencils): row position t has columns
    // sell_node[t] + pat_off[pat_id[t] * kPatLen + k], k < rowlen[t]
    std::vector<uint8_t> pat_id;         // [n_nodes], empty without stencils
    std::vector<int32_t> pat_off;        // [n_pat * kPatLen]
    int n_pat = 0;
    // upper-only layout (build_sell_sym, FP32): row i stores its blocks
    // (i, c >= i); the lower block (i, j < i) is the transpose of the stored
    // (j, i), at position q of row j.  Transposed stencils list, per row, the
    // lower neighbours in ascending order as (offset j - i, q) pairs;
    // bsr_to_sell holds -2 - slot for a lower block, el_blk -1.
    bool sym = false;
    std::vector<uint8_t> tpat_id;        // [n_nodes]
    std::vector<int32_t> tpat;           // [n_tpat * kPatLen * 2] (offset, q)
    std::vector<int32_t> tpat_len;       // [n_tpat]
    int n_tpat = 0;
};

// the same on the device
struct SellDev {
    int64_t n_sell = 0;
    int64_t *slice_base = nullptr, *diag_blk = nullptr;
    int32_t *sell_col = nullptr, *rowlen = nullptr, *sell_node = nullptr, *el_blk = nullptr;
    uint8_t *pat_id = nullptr;           // row stencils, null without
    int32_t *pat_off = nullptr;
    int n_pat = 0;
    bool sorted = false;                 // the FP32 layouts use slot pairs, the FP64 layouts do not
    bool sym = false;                    // upper-only layout (always with row and transposed stencils)
    uint8_t *tpat_id = nullptr;
    int2 *tpat = nullptr;                // [n_tpat * kPatLen] (offset, q)
    int32_t *tpat_len = nullptr;
};

// buffers of the mixed-precision solve (FP32 tangent and CG)
struct MixedBuffers {
    float *dphi = nullptr;        // [n_el*nq*2*nn]
    float *K = nullptr;           // [sell.n_sell*4]
    SellLayout sell;              // node-ordered rows (the FP32 SpMV is gather-bound)
    SellDev dsell;
    // the upper-only layout, used with row stencils where it can be built
    // (structured grids): half the tangent bytes of `sell`
    float *Ks = nullptr;          // [sym.n_sell*4]
    SellLayout sym;
    SellDev dsym;
    bool have_sym = false;
    float *dinv = nullptr;        // [neq]
    float *binv = nullptr;        // [n_nodes*4] block-Jacobi inverses
    float *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr;
    float *part = nullptr;        // 2 partial arrays
    float *strain32 = nullptr, *sigw32 = nullptr;   // [3][n_ip] FP32 residual (ipfem_set_residual_precision)
    float *fe32 = nullptr;                          // [n_el][nd]
    // element blocks of the FP32 residual kernels in tiles of kTile32
    // elements: [tile][d][n][element of the tile][q], the point index padded
    // to the odd stride nq | 1, the last tile and the padding zero
    float *dphiT = nullptr;
    CGScalarsT<float> *sc = nullptr;
    CGScalarsT<float> *h_sc = nullptr;   // pinned
    cudaGraphExec_t exec = nullptr;
};

// Host result of the setup: everything derived from the mesh (colouring,
// dof map, nodal 2x2 block pattern in SELL-32 layout, colour incidence).
struct Setup {
    int32_t n_el = 0, n_nodes = 0, neq = 0, n_colors = 0;
    int32_t order = 2, nn = 9, nq = 9, nd = 18;   // element order; connects, points, dofs per element
    int64_t n_ip = 0;
    std::vector<double> dphi;            // [n_el*nq*2*nn] ((e*nq+q)*2+d)*nn+n
    std::vector<double> weight;          // [n_ip]
    std::vector<int32_t> dofs;           // [n_el*nd]
    std::vector<int32_t> el_color;       // [n_el]
    std::vector<int32_t> color_ptr;      // [n_colors+1]
    std::vector<int32_t> color_els;      // [n_el]
    std::vector<int32_t> inc;            // [n_colors*n_nodes] e*nn+local node or -1
    // nodal block pattern (rows ascending, columns ascending)
    int64_t n_blocks = 0;
    std::vector<int64_t> row_ptr;        // [n_nodes+1]
    std::vector<int32_t> col;            // [n_blocks]
    // SELL-32 layout of the same blocks for the FP64 tangent: rows sorted by
    // length inside each kRedBlock window (the FP64 SpMV is FP64-pipe-bound)
    SellLayout sell;
    std::vector<uint8_t> fixed;          // [neq]
    std::vector<double> f0, df;          // [neq]
    std::vector<double> mat;             // [5*n_el] SoA: c, sinphi, cosphi, tanphi, sinpsi
    ElasticConstH el{};
    double eps_p0[4] = {0, 0, 0, 0};     // in-situ plastic strain seed xx, xy, yy, zz
    double sigma0[4] = {0, 0, 0, 0};
};

// builds the setup; returns an empty string or an error message
std::string build_setup(const ipfem_mesh *mesh, const ipfem_material *mat, Setup &s);
// d(phi)/dx, d(phi)/dy and w|detJ| at the (p+1)^2 Gauss points of order-p
// Lagrange elements with bilinear geometry from their 4 vertex connects, or,
// where shape[e] = 1, of triangles from their 3 (host, threaded)
void element_blocks_dphi(int order, int64_t n_el, const int32_t *connects, const double *node_xy, double *dphi,
                         double *weight, const uint8_t *shape = nullptr);
// an order-p triangle in the block shape of the order-p quadrilateral (ghost columns zero)
void tri_element_dphi(int p, const double *X, const double *Y, double *dphi, double *w);
int32_t greedy_coloring_nn(int32_t n_el, int32_t n_nodes, int32_t nn, const int32_t *connects, int32_t *el_color);
// SELL-32 layout of s's block pattern; sorted: rows by length inside each
// kRedBlock-node window (stable, longest first)
std::string build_sell(const Setup &s, bool sorted, bool pair, SellLayout &L);

// slot of block k of row position t
inline int64_t sell_slot(const SellLayout &L, int64_t t, int64_t k)
{
    return L.pair ? L.slice_base[t / 32] + 64 * (k >> 1) + 2 * (t % 32) + (k & 1)
                  : L.slice_base[t / 32] + 32 * k + t % 32;
}

#ifdef __CUDACC__
// the same on the device, split into the row's first slot (slice start
// slice0, lane = t % 32) and the offset of its block k
template <bool PAIR>
__device__ __forceinline__ int64_t sell_row0(int64_t slice0, int lane)
{
    return slice0 + (PAIR ? 2 * lane : lane);
}
template <bool PAIR>
__device__ __forceinline__ int64_t sell_koff(int k)
{
    return PAIR ? 64 * (int64_t)(k >> 1) + (k & 1) : 32 * (int64_t)k;
}
// upper-only FP32 layout (rows in node order, slot pairs): the slot of the
// block at position q of row j, i.e. the stored twin of a lower block
__device__ __forceinline__ int64_t sym_twin_slot(const int64_t *__restrict__ slice_base, int32_t j, int q)
{
    return sell_row0<true>(__ldg(&slice_base[j >> 5]), j & 31) + sell_koff<true>(q);
}
// a 2x2 block (row-major float4) transposed
__device__ __forceinline__ float4 transpose4(float4 b)
{
    return make_float4(b.x, b.z, b.y, b.w);
}
#endif
void build_row_stencils(SellLayout &L);
// the upper-only FP32 layout with its row and transposed stencils; returns an
// empty string, or why it cannot be built (the full layout is used then)
std::string build_sell_sym(const Setup &s, SellLayout &L);
void elastic_constants(double E, double nu, ElasticConstH &el);
// message returned by ipfem_last_error(NULL) on the calling thread
void set_thread_error(const std::string &msg);

}  // namespace ipfem

struct NewtonState {
    ipfem_solve_opts opts{};
    int32_t step = 0, step_end = 0, it = 0;
    int open = 0, active = 0, all_converged = 1;
    double r0 = 0.0, rn = 0.0;
    double alpha = 1.0;           // modified-Thomas acceleration factor of the open load step
    int have_k = 0;               // a tangent has been assembled since newton_begin
    double eta = 0.0;             // inner tolerance of the last solve of the open load step
    double rn_prev = 0.0;         // |R| before the last Newton iteration
    int have_prev = 0;            // d_u_prev holds the solution of the previous accepted load step
    double r_pred = 0.0;          // |R| at the predicted start of the open load step
};
// adaptive inner tolerance (ipfem_set_inner_tolerance)
struct InnerTolerance {
    int mode = 0;
    double gamma = 0.9, alpha = 2.0, eta_min = 1e-5, eta_max = 0.1;
};

namespace ipfem {
// learned preconditioner (per-node MLP -> symmetric 3x3-patch operator) and
// its training state
struct MlpBuffers {
    float *params = nullptr;      // FP32 master: W1[32][128] b1[128] W2[128][128] b2[128] W3[128][20] b3[20]
    float *grads = nullptr, *m = nullptr, *v = nullptr;
    void *w1t = nullptr, *w2t = nullptr, *w3t = nullptr;   // BF16 [128][32], [128][128], [24][128] (n, k)
    int32_t *slot = nullptr;      // [9][n_nodes] FP32-tangent slot of block (i, nbr(i, k)) or -1
    int32_t *pslot = nullptr;     // [25][n_nodes] slot of block (nbr(i, k), nbr(i, l)), k, l < 5, or -1
    int32_t *slot_s = nullptr, *pslot_s = nullptr;   // the same codes for the upper-only layout (-2 - slot: transposed)
    float nf = 0.f;               // number of free dofs
    float *X = nullptr;           // [n_nodes][32] features of the current tangent
    float *O = nullptr;           // [n_nodes][20] network output
    float *M = nullptr;           // [5][n_nodes][4] triangular factor G (M = sigma G^T G sigma)
    float *y = nullptr;           // [neq] first stencil pass of the preconditioner
    void *Gh = nullptr;           // [5][n_nodes] BF16 copy of G (4 values per block) for the solves
    float *p2 = nullptr;          // [neq] second search-direction buffer of the fused flexible CG
    float *r_old = nullptr;       // flexible-CG previous residual
    float *loss = nullptr, *scal = nullptr;
    // training scratch (allocated by the first gradient pass)
    float *H1 = nullptr, *H2 = nullptr, *dH1 = nullptr, *dH2 = nullptr, *dN = nullptr, *part = nullptr;
    float *vec = nullptr;         // 7 x neq
    int32_t gr = 0, gt = 0;       // structured node grid (gr x gt)
    int64_t adam_t = 0;
    bool ready = false, op_valid = false;
};
constexpr int kMlpParams = 32 * 128 + 128 + 128 * 128 + 128 + 128 * 20 + 20;
constexpr int kOffW1 = 0, kOffB1 = 4096, kOffW2 = 4224, kOffB2 = 20608, kOffW3 = 20736, kOffB3 = 23296;
static_assert(kOffB3 + 20 == kMlpParams, "parameter layout");
}  // namespace ipfem

struct ipfem_ctx {
    int device = -1;
    cudaStream_t stream = nullptr;
    ipfem::Setup s;
    std::string err;
    double load_factor = 0.0;
    int update_mem = 0;
    // device: setup
    double *d_dphi = nullptr, *d_weight = nullptr, *d_mat = nullptr, *d_f0 = nullptr, *d_df = nullptr;
    double *d_lin = nullptr;             // [neq] f0 + load_factor * df (the reference's fRhsLinear)
    int32_t *d_dofs = nullptr, *d_color_els = nullptr, *d_inc = nullptr;
    uint8_t *d_fixed = nullptr;
    ipfem::SellDev dsell;                // FP64 tangent layout
    // device: tangent
    double *d_K = nullptr, *d_dinv = nullptr;
    double *d_binv = nullptr;             // [n_nodes*4] block-Jacobi inverses (IPFEM_PREC_BLOCK_JACOBI)
    // device: integration-point state {xx, xy, yy, zz} SoA
    double *d_eps_p = nullptr, *d_sigma = nullptr, *d_alpha = nullptr;
    int8_t *d_mtype = nullptr;
    // device: work
    double *d_u = nullptr, *d_rhs = nullptr, *d_strain = nullptr, *d_sigma_w = nullptr, *d_dep = nullptr;
    double *d_fe = nullptr;
    double *d_x = nullptr, *d_r = nullptr, *d_z = nullptr, *d_p = nullptr, *d_q = nullptr, *d_b = nullptr;
    double *d_part = nullptr;            // 3 partial arrays of n_red each
    int64_t n_red = 0;                   // number of reduction blocks
    ipfem::CGScalars *d_sc = nullptr;
    unsigned *d_counters = nullptr;      // last-block tickets
    double *d_dotres = nullptr;          // results of standalone dots
    int newton_accel = 0;                // 1: modified-Thomas accelerated Newton (main.cpp:194-224)
    int newton_tangent = 0;              // 1: initial stiffness (tangent of the first assembly kept)
    double *d_acc = nullptr;             // [neq] alpha * du of the accelerated step
    int *d_err = nullptr;                // device error word (wait timeouts)
    ipfem::CGScalars *h_sc = nullptr;    // pinned
    double *h_pin = nullptr;             // pinned scalars
    cudaGraphExec_t cg_exec = nullptr;
    int cg_batch = 0;
    bool tangent_valid = false;
    NewtonState ns;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    bool ev_ready = false;
    uint64_t launches = 0;               // kernels launched through this context
    int precision = 0;                   // IPFEM_PLAIN_FP64 or IPFEM_MIXED
    ipfem::MixedBuffers mx;
    int preconditioner = 0;              // IPFEM_PREC_JACOBI, IPFEM_PREC_MLP or IPFEM_PREC_BLOCK_JACOBI
    int row_stencils = 1;                // SpMVs read row stencils where the layout has them
    ipfem::MlpBuffers mlp;
    cudaGraphExec_t fcg_exec = nullptr;
    int64_t fcg_fallbacks = 0;
    FILE *iter_log = nullptr;            // JSON-lines record of the Newton iterations (ipfem_set_iteration_log)
    int res32 = 0;                       // FP32 residual evaluations in IPFEM_MIXED (ipfem_set_residual_precision)
    int res32_active = 0;                // the residuals being evaluated now are FP32
    double res32_switch = 1e-5;          // |R| / |R0| below which a load step refines with FP64 residuals
    InnerTolerance inner;                // inner tolerance of the Newton iterations
    int predictor = 0;                   // secant predictor at the start of each load step
    int consistent_tangent = 0;          // consistent spectral tangent (ipfem_set_consistent_tangent)
    int spectral_mode = 0;               // 1: closed-form plane-strain decomposition (ipfem_set_spectral_mode)
    double *d_u_prev = nullptr;          // [neq] solution of the previous accepted load step (predictor)
};

// ---- kernel launchers (implemented in the .cu files) ----
namespace ipfem {
// whether the SpMVs over layout L read its row stencils
inline bool use_row_stencils(const ipfem_ctx *c, const SellDev &L)
{
    return c->row_stencils != 0 && L.n_pat > 0 && L.pat_id != nullptr;
}
// whether the FP32 tangent lives in the upper-only layout (with row stencils on)
inline bool use_sym32(const ipfem_ctx *c)
{
    return c->mx.have_sym && c->row_stencils != 0;
}
// the FP32 tangent's active layout and values
inline const SellDev &fp32_layout(const ipfem_ctx *c)
{
    return use_sym32(c) ? c->mx.dsym : c->mx.dsell;
}
inline float *fp32_values(const ipfem_ctx *c)
{
    return use_sym32(c) ? c->mx.Ks : c->mx.K;
}

void launch_gather_strain(ipfem_ctx *c, const double *d_u, double *d_strain);
void launch_compute_sigma(ipfem_ctx *c, int update_mem, const double *d_strain, double *d_sigma_w, double *d_dep);
void launch_stress_residual(ipfem_ctx *c, const double *d_sigma_w, double *d_fe);
// d_lin = f0 + c->load_factor * df, after every change of the load factor
void launch_load_vector(ipfem_ctx *c);
void launch_color_reduce(ipfem_ctx *c, const double *d_fe, int with_load, double *d_res);
// the FP32 residual of IPFEM_MIXED_RES32: FP32 gather, FP64 point update on
// FP32 strains, FP32 scatter and colour sums (the load added in FP64)
// elements per tile of the FP32 residual's interleaved blocks (one per lane)
constexpr int kTile32 = 32;
// fills c->mx.dphiT (allocated: n_tiles * kTile32 * 2*nn * (nq | 1) floats) from the FP64 blocks
void launch_tile_blocks32(ipfem_ctx *c);
void launch_gather_strain32(ipfem_ctx *c, const double *d_u, float *d_strain);
void launch_compute_sigma32(ipfem_ctx *c, int update_mem, const float *d_strain, float *d_sigma_w, double *d_dep);
void launch_stress_residual32(ipfem_ctx *c, const float *d_sigma_w, float *d_fe);
void launch_color_reduce32(ipfem_ctx *c, const float *d_fe, int with_load, double *d_res);
void launch_stiffness(ipfem_ctx *c);
void launch_cg_init(ipfem_ctx *c, const double *d_b, double rtol, int max_it);
void launch_cg_iteration(ipfem_ctx *c);
void launch_cg_spmv_only(ipfem_ctx *c);
void launch_dot(ipfem_ctx *c, const double *a, const double *b, double *d_out);
void launch_axpy_u(ipfem_ctx *c, double *d_u, const double *d_du);
// u <- u + ratio (u - u_prev), u_prev <- the old u
void launch_predict(ipfem_ctx *c, double *d_u, double *d_u_prev, double ratio);
void launch_scale_add(ipfem_ctx *c, double *d_u, const double *d_x, double alpha, double *d_t);
void launch_fp64_probe(ipfem_ctx *c, double *d_out, int grid, int iters);
void launch_stiffness32(ipfem_ctx *c);
// recomputes the Jacobi (and, when allocated, block-Jacobi) inverses of the current tangent
void launch_jacobi(ipfem_ctx *c);
void launch_cg32_init(ipfem_ctx *c, const double *d_b, double scale, float rtol, int max_it);
void launch_cg32_iteration(ipfem_ctx *c);
void launch_cg32_spmv_only(ipfem_ctx *c);

void launch_add_scaled32(ipfem_ctx *c, double *d_u, const float *x, double scale);
// solver drivers (capi.cpp, capi_mlp.cu)
ipfem_status check_device(ipfem_ctx *c);
ipfem_status cg_device(ipfem_ctx *c, const double *d_b, double rtol, int max_it, int *iters);
ipfem_status cg32_device(ipfem_ctx *c, const double *d_b, double scale, double rtol, int max_it, int *iters);
ipfem_status fcg_device(ipfem_ctx *c, const double *d_b, double scale, double rtol, int max_it, int *iters,
                        int *fell_back);
ipfem_status dot_host(ipfem_ctx *c, const double *a, const double *b, double *out);
// learned preconditioner (k_mlp.cu)
void mlp_pack_weights(ipfem_ctx *c);
cudaError_t mlp_configure();
void launch_patch_features(ipfem_ctx *c, float *d_X);
void launch_patch_net(ipfem_ctx *c, int64_t rows, const float *d_X, float *d_O);
// tcgen05 network kernel (k_net_tc.cu)
cudaError_t net_tc_configure();
// C = op(A) op(B) on tcgen05 (BF16 operands, FP32 accumulation), split K over gridDim.z
void launch_gemm_tc(ipfem_ctx *c, int M, int N, int K, const float *A, int lda, int transA, const float *B, int ldb,
                    int transB, float *C, int ldc, int kchunk, int splits, float *colsum = nullptr);
void launch_patch_net_tc(ipfem_ctx *c, int64_t rows, const float *d_X, float *d_O, float *d_H1 = nullptr,
                         float *d_H2 = nullptr);
void launch_patch_net_bwd_tc(ipfem_ctx *c, int64_t rows, const float *d_dO, const float *d_H1, const float *d_H2,
                             float *d_dH2, float *d_dH1);
void launch_patch_operator(ipfem_ctx *c);
void launch_fcg_init(ipfem_ctx *c, const double *d_b, double scale, float rtol, int max_it);
void launch_fcg_iteration(ipfem_ctx *c, int par);
size_t patch_part_floats(int64_t n_nodes);
void patch_learn_grad(ipfem_ctx *c, const float *d_r, const float *d_e, int P, float wk, float wp);
void mlp_adam_step(ipfem_ctx *c, float lr);
}  // namespace ipfem
