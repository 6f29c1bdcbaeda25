// Learned preconditioner: a per-node MLP (32 -> 128 -> 128 -> 20) that maps the
// FP32 tangent around a node to its block row of a sparse triangular factor
// G, used as M = diag(sigma) G^T G diag(sigma) inside flexible CG.  No
// counterpart in the reference.
//
// Node i = b*gr + a of a structured node grid; patch position k = 3*(db+1) +
// (da+1) for da, db in {-1, 0, 1} (k = 4 is the node itself, 8 - k the mirror).
// With sigma = sqrt(Dinv) per dof (0 on Dirichlet dofs) and f = (sigma > 0):
//   features  X_i[4m + 2p + q] = K_ij[p][q] sigma_i[p] sigma_j[q] for the 8
//             neighbours j (m-th non-centre position), 0 outside the grid or
//             where the couplings are absent from the tangent;
//   network   O_i[20] = W3^T relu(W2^T relu(W1^T X_i + b1) + b2) + b3;
//   factor    G_ik = O_i[4k..4k+3] (row-major 2x2) for the lower neighbours
//             k = 0..3, G_i4 = [[exp(O_i[16]), 0], [O_i[17], exp(O_i[18])]],
//             each entry times f_i[p] f_j[q];
//   operator  M = diag(sigma) G^T G diag(sigma),
// symmetric positive definite on the free dofs by construction (G is block
// triangular in node order with a positive diagonal) and Jacobi for O = 0.
// The network runs once per tangent; each CG iteration applies G and G^T
// (two 5-block stencil passes).  Training minimises the log of Kaporin's
// condition number of M K plus the residual of the plain solver's
// (residual, increment) pairs.
//
// The network runs on the 5th-generation tensor cores (tcgen05.mma, TMEM
// accumulators, BF16 operands, FP32 accumulation; k_net_tc.cu): inference and
// the training forward in k_patch_net_tc, the backward of the hidden layers in
// k_patch_net_bwd_tc, the split-K weight gradients in k_gemm_tc.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>

#include "ipfem_internal.h"
#include "ldhint.cuh"
#include "pdl.cuh"

namespace ipfem {

constexpr unsigned FULLM = 0xffffffffu;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

// out[i] = sum_z part[z*n + i] (split-K partials): CTA x sums columns
// 32x .. 32x+31, its 8 warps split z = w, w+8, ... and are added in warp order
__global__ void __launch_bounds__(256) k_sum_splits(int64_t n, int splits, const float *__restrict__ part,
                                                    float *__restrict__ out)
{
    __shared__ float s[8][33];
    const int64_t i = blockIdx.x * (int64_t)32 + (threadIdx.x & 31);
    const int w = threadIdx.x >> 5;
    float a = 0.f;
    if (i < n)
        for (int z = w; z < splits; z += 8) a += part[(size_t)z * n + i];
    s[w][threadIdx.x & 31] = a;
    __syncthreads();
    if (w == 0 && i < n) {
        float t = 0.f;
#pragma unroll
        for (int k = 0; k < 8; k++) t += s[k][threadIdx.x];
        out[i] = t;
    }
}

// Adam on the FP32 parameter vector
__global__ void k_adam(int n, float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// ------------------------------------------------------------ node grid
struct GridInfo {
    int32_t gr, gt;
};

// neighbour of node i at patch position k, or -1 outside the grid
__device__ __forceinline__ int32_t patch_nbr(int32_t i, int k, GridInfo G)
{
    const int a = i % G.gr + k % 3 - 1, b = i / G.gr + k / 3 - 1;
    if (a < 0 || b < 0 || a >= G.gr || b >= G.gt) return -1;
    return b * G.gr + a;
}

__device__ __forceinline__ float2 sqrt2(float2 d)
{
    return make_float2(sqrtf(d.x), sqrtf(d.y));
}

// block (i, j) of the FP32 tangent from its slot code: s >= 0 the stored
// block, s <= -2 the transpose of the stored twin -2 - s (the lower blocks of
// the upper-only layout); -1 (no block) is the caller's case
__device__ __forceinline__ float4 tangent_block(const float4 *__restrict__ K, int32_t s)
{
    return s >= 0 ? K[s] : transpose4(K[-2 - s]);
}

// features X[n][32] from the FP32 tangent: scaled couplings to the 8
// neighbours (slot[k][n] = slot code of block (i, nbr(i, k)), -1 for none)
__global__ void __launch_bounds__(256) k_patch_features(int32_t n, GridInfo G, const float4 *__restrict__ K,
                                                        const int32_t *__restrict__ slot,
                                                        const float2 *__restrict__ dinv, float *__restrict__ X)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 si = sqrt2(dinv[i]);
    float4 *xo = reinterpret_cast<float4 *>(X + (int64_t)i * 32);
    int m = 0;
#pragma unroll
    for (int k = 0; k < 9; k++) {
        if (k == 4) continue;
        const int32_t s = slot[(int64_t)k * n + i];
        float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
        if (s != -1) {
            const float4 blk = tangent_block(K, s);
            const float2 sj = sqrt2(dinv[patch_nbr(i, k, G)]);
            f = make_float4(blk.x * si.x * sj.x, blk.y * si.x * sj.y, blk.z * si.y * sj.x, blk.w * si.y * sj.y);
        }
        xo[m++] = f;
    }
}

// ------------------------------------------------ network output width
// The inference network itself runs on the tcgen05 tensor cores (k_net_tc.cu).
constexpr int NOUT = 20, NOUTP = 24;    // outputs per node; W3^T rows stored (padded to 24)

__device__ __forceinline__ float2 free2(float2 d)
{
    return make_float2(d.x > 0.f ? 1.f : 0.f, d.y > 0.f ? 1.f : 0.f);
}

constexpr int NTRI = 5;          // factor blocks per node: k = 0..3 and the node (k = 4)

// the log-diagonal outputs are clamped to [-30, 30] before exp (a network far
// outside its training data cannot overflow the factor)
__device__ __forceinline__ float clamp_log(float o)
{
    return fminf(fmaxf(o, -30.f), 30.f);
}

// BF16 copy of a factor block for the solves (FP32 range, so no overflow for
// any finite factor; the same rounded G enters both passes, so M stays SPD)
__device__ __forceinline__ uint2 half4(float4 v)
{
    return make_uint2(pack_bf16(v.x, v.y), pack_bf16(v.z, v.w));
}

__device__ __forceinline__ float4 load_g(const float4 *__restrict__ g, int64_t idx)
{
    return __ldg(&g[idx]);
}

// four BF16 values (one 2x2 factor block) widened to FP32
__device__ __forceinline__ float4 bf16x4(uint2 u)
{
    const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&u.x));
    const float2 b = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&u.y));
    return make_float4(a.x, a.y, b.x, b.y);
}

__device__ __forceinline__ float4 load_g(const uint2 *__restrict__ g, int64_t idx)
{
    return bf16x4(__ldg(&g[idx]));
}

// G[k][i] (float4, row-major 2x2, k = 0..4) from the network output O[n][20],
// and its BF16 copy Gh for the solves when given
__global__ void __launch_bounds__(256) k_tri_build(int32_t n, GridInfo G, const float *__restrict__ O,
                                                   const float2 *__restrict__ dinv, float4 *__restrict__ Gm,
                                                   uint2 *__restrict__ Gh)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 fi = free2(dinv[i]);
    const float *oi = O + (int64_t)i * NOUT;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int32_t j = patch_nbr(i, k, G);
        float4 gk = make_float4(0.f, 0.f, 0.f, 0.f);
        if (j >= 0) {
            const float2 fj = free2(dinv[j]);
            gk = make_float4(oi[4 * k] * fi.x * fj.x, oi[4 * k + 1] * fi.x * fj.y, oi[4 * k + 2] * fi.y * fj.x,
                             oi[4 * k + 3] * fi.y * fj.y);
        }
        Gm[(int64_t)k * n + i] = gk;
        if (Gh) Gh[(int64_t)k * n + i] = half4(gk);
    }
    const float4 g4 = make_float4(expf(clamp_log(oi[16])) * fi.x, 0.f, oi[17] * fi.y * fi.x,
                                  expf(clamp_log(oi[18])) * fi.y);
    Gm[(int64_t)4 * n + i] = g4;
    if (Gh) Gh[(int64_t)4 * n + i] = half4(g4);
}

// y_i = sum_k G_ik (sigma * x)_nbr(i,k)
template <class GT>
__device__ __forceinline__ float2 tri_mul(int32_t i, int32_t n, GridInfo G, const GT *__restrict__ Gm,
                                          const float2 *__restrict__ dinv, const float2 *__restrict__ x)
{
    float2 y = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < NTRI; k++) {
        const int32_t j = patch_nbr(i, k, G);
        if (j < 0) continue;
        const float4 m = load_g(Gm, (int64_t)k * n + i);
        const float2 s = sqrt2(__ldg(&dinv[j])), v = __ldg(&x[j]);
        const float vx = s.x * v.x, vy = s.y * v.y;
        y.x = fmaf(m.x, vx, fmaf(m.y, vy, y.x));
        y.y = fmaf(m.z, vx, fmaf(m.w, vy, y.y));
    }
    return y;
}

// z_j = sigma_j * sum_k G_{i,k}^T y_i over the nodes i = nbr(j, 8-k) that
// hold j at position k (gather form of G^T)
template <class GT>
__device__ __forceinline__ float2 trit_mul(int32_t j, int32_t n, GridInfo G, const GT *__restrict__ Gm,
                                           const float2 *__restrict__ dinv, const float2 *__restrict__ y)
{
    float2 z = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < NTRI; k++) {
        const int32_t i = patch_nbr(j, 8 - k, G);
        if (i < 0) continue;
        const float4 m = load_g(Gm, (int64_t)k * n + i);
        const float2 v = __ldg(&y[i]);
        z.x = fmaf(m.x, v.x, fmaf(m.z, v.y, z.x));
        z.y = fmaf(m.y, v.x, fmaf(m.w, v.y, z.y));
    }
    const float2 s = sqrt2(dinv[j]);
    return make_float2(s.x * z.x, s.y * z.y);
}

// y = G (sigma * r); skipped once the solve is done when sc is given
template <class GT>
__global__ void __launch_bounds__(256) k_tri_first(int32_t n, GridInfo G, const GT *__restrict__ Gm,
                                                   const float2 *__restrict__ dinv, const float2 *__restrict__ r,
                                                   float2 *__restrict__ y, const CGScalarsT<float> *sc)
{
    if (sc && *reinterpret_cast<const volatile int *>(&sc->done)) return;
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = tri_mul(i, n, G, Gm, dinv, r);
}

// z = sigma * (G^T y)
__global__ void __launch_bounds__(256) k_tri_second(int32_t n, GridInfo G, const float4 *__restrict__ Gm,
                                                    const float2 *__restrict__ dinv, const float2 *__restrict__ y,
                                                    float2 *__restrict__ z)
{
    const int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) z[j] = trit_mul(j, n, G, Gm, dinv, y);
}

// ------------------------------------------------------ flexible CG (FP32)
// Reductions: warp tree, in-order sum over the CTA's warps, last CTA.
__device__ __forceinline__ float wsum(float v)
{
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v = v + __shfl_down_sync(FULLM, v, off);
    return v;
}

template <int NV>
__device__ bool fcg_partials(const float (&v)[NV], float *part, int64_t n_part, unsigned *ticket)
{
    __shared__ float ws[NV][32];
    __shared__ int s_last;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        const float t = wsum(v[k]);
        if (lane == 0) ws[k][w] = t;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            float a = 0.f;
            for (int i = 0; i < nw; i++) a = a + ws[k][i];
            part[k * n_part + blockIdx.x] = a;
        }
        __threadfence();
        s_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    return s_last != 0;
}

template <int NV>
__device__ void fcg_final(const float *part, int64_t n_part, float (&out)[NV])
{
    __shared__ float ws[NV][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        float a = 0.f;
        for (int64_t i = threadIdx.x; i < n_part; i += blockDim.x) a = a + __ldcg(&part[k * n_part + i]);
        a = wsum(a);
        if (lane == 0) ws[k][w] = a;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            float a = 0.f;
            for (int i = 0; i < nw; i++) a = a + ws[k][i];
            out[k] = a;
        }
    }
}

// x = 0, p = 0, r = b*scale (FP64 -> FP32), r_old = 0; b.b
__global__ void __launch_bounds__(256) k_fcg_init(int32_t n_nodes, const double *__restrict__ b, double scale,
                                                  float *__restrict__ x, float *__restrict__ r, float *__restrict__ p,
                                                  float *__restrict__ r_old, float *part, int64_t n_part,
                                                  unsigned *ticket, CGScalarsT<float> *sc, float rtol, int max_it)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float v[1] = {0.f};
    if (i < n_nodes) {
        const double2 bb = reinterpret_cast<const double2 *>(b)[i];
        const float2 rr = make_float2((float)(bb.x * scale), (float)(bb.y * scale));
        reinterpret_cast<float2 *>(r)[i] = rr;
        reinterpret_cast<float2 *>(r_old)[i] = make_float2(0.f, 0.f);
        reinterpret_cast<float2 *>(x)[i] = make_float2(0.f, 0.f);
        reinterpret_cast<float2 *>(p)[i] = make_float2(0.f, 0.f);
        v[0] = fmaf(rr.y, rr.y, rr.x * rr.x);
    }
    if (fcg_partials<1>(v, part, n_part, ticket)) {
        float o[1];
        fcg_final<1>(part, n_part, o);
        if (threadIdx.x == 0) {
            sc->bb = o[0];
            sc->rr = o[0];
            sc->thr = (rtol * rtol) * o[0];
            sc->rz = 0.f;
            sc->beta = 0.f;
            sc->iters = 0;
            sc->status = 0;
            sc->max_it = max_it;
            sc->rr_best = o[0];
            sc->it_best = 0;
            sc->fallback = 0;
            sc->done = (o[0] == 0.f) ? 1 : (max_it <= 0 ? 1 : 0);
            if (o[0] != 0.f && max_it <= 0) sc->status = IPFEM_NONCONVERGED;
            *ticket = 0u;
        }
    }
}

// z = M r = sigma * (G^T y) with y = G (sigma * r) from k_tri_first; partial
// r.z and r_old.z; last CTA: Polak-Ribiere beta = (r.z - r_old.z) / rz_prev
// (clipped at 0), rz = r.z
__global__ void __launch_bounds__(256) k_tri_precond(int32_t n, GridInfo G, const uint2 *__restrict__ Gm,
                                                     const float2 *__restrict__ dinv, const float2 *__restrict__ y,
                                                     const float *__restrict__ r, const float *__restrict__ r_old,
                                                     float *__restrict__ z, float *part, int64_t n_part,
                                                     unsigned *ticket, CGScalarsT<float> *sc)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    // r_old (not written by the update pass) before the wait; y, r and the
    // flag after it
    float2 ro = make_float2(0.f, 0.f);
    if (i < n) ro = reinterpret_cast<const float2 *>(r_old)[i];
    pdl_wait();
    pdl_launch_dependents();
    if (*reinterpret_cast<volatile int *>(&sc->done)) return;
    float v[2] = {0.f, 0.f};
    if (i < n) {
        const float2 zz = trit_mul(i, n, G, Gm, dinv, y);
        reinterpret_cast<float2 *>(z)[i] = zz;
        const float2 rr = reinterpret_cast<const float2 *>(r)[i];
        v[0] = fmaf(rr.y, zz.y, rr.x * zz.x);
        v[1] = fmaf(ro.y, zz.y, ro.x * zz.x);
    }
    if (fcg_partials<2>(v, part, n_part, ticket)) {
        float out[2];
        fcg_final<2>(part, n_part, out);
        if (threadIdx.x == 0) {
            const float rz = out[0], cross = out[1];
            float beta = (sc->rz > 0.f) ? (rz - cross) / sc->rz : 0.f;
            if (!(beta > 0.f)) beta = 0.f;
            sc->beta = beta;
            sc->rz = rz;
            if (!(rz > 0.f)) {          // M r is not a descent direction
                sc->done = 1;
                sc->status = kStatusFallback;
            }
            *ticket = 0u;
        }
    }
}

// ----------------------------------------- fused flexible-CG iteration (FP32)
// One iteration = k_fcg_spmv, k_fcg_update_first, k_tri_precond (factor in
// BF16), with the
// search direction and the residual double-buffered (the caller alternates
// the buffers): the p-update of the previous iteration is formed on the fly
// inside the SpMV, the x/r update inside the first factor pass.

// p_new = z + beta p_old (the owner stores it, gatherers form it for their
// columns), q = K p_new, partials of p_new.q; last CTA: alpha = rz / pq.
// Node-ordered SELL rows; the tangent and its column indices are streamed
// (evict-first) so that z and p_old stay in L2.
template <bool PAT>
__global__ void __launch_bounds__(256, 8) k_fcg_spmv(int32_t n, const int64_t *__restrict__ slice_base,
                                                  const int32_t *__restrict__ rowlen, const int32_t *__restrict__ scol,
                                                  const uint8_t *__restrict__ pat_id,
                                                  const int32_t *__restrict__ pat_off,
                                                  const float4 *__restrict__ K, const uint8_t *__restrict__ fixed,
                                                  const float2 *__restrict__ z, const float2 *__restrict__ p_old,
                                                  float2 *__restrict__ p_new, float2 *__restrict__ q, float *part,
                                                  int64_t n_part, unsigned *ticket, CGScalarsT<float> *sc)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    // row metadata before the wait; z, beta and the flag (written by the
    // preconditioner pass) after it
    int64_t base = 0;
    int len = 0, pb = 0;
    if (i < n) {
        base = sell_row0<true>(__ldg(&slice_base[i >> 5]), i & 31);
        len = __ldg(&rowlen[i]);
        if (PAT) pb = (int)__ldg(&pat_id[i]) * kPatLen;
    }
    pdl_wait();
    pdl_launch_dependents();
    if (*reinterpret_cast<volatile int *>(&sc->done)) return;
    const float beta = *reinterpret_cast<volatile float *>(&sc->beta);
    float v[1] = {0.f};
    if (i < n) {
        const uint64_t keep = l2_policy_keep();
        float y0 = 0.f, y1 = 0.f;
#pragma unroll 4
        for (int k = 0; k < len; k++) {
            const int64_t s = base + sell_koff<true>(k);
            const int32_t c = PAT ? i + __ldg(&pat_off[pb + k]) : __ldcs(&scol[s]);
            const float4 a = __ldcs(&K[s]);
            const float2 zz = ld_keep(&z[c], keep), pp = ld_keep(&p_old[c], keep);
            const float px = fmaf(beta, pp.x, zz.x), py = fmaf(beta, pp.y, zz.y);
            y0 = fmaf(a.y, py, fmaf(a.x, px, y0));
            y1 = fmaf(a.w, py, fmaf(a.z, px, y1));
        }
        if (fixed[2 * (int64_t)i]) y0 = 0.f;
        if (fixed[2 * (int64_t)i + 1]) y1 = 0.f;
        q[i] = make_float2(y0, y1);
        const float2 zi = z[i], pi = p_old[i];
        const float2 pn = make_float2(fmaf(beta, pi.x, zi.x), fmaf(beta, pi.y, zi.y));
        p_new[i] = pn;
        v[0] = fmaf(pn.y, y1, pn.x * y0);
    }
    if (fcg_partials<1>(v, part, n_part, ticket)) {
        float o[1];
        fcg_final<1>(part, n_part, o);
        if (threadIdx.x == 0) {
            const float pq = o[0];
            sc->pq = pq;
            if (!(pq > 0.f)) {
                sc->done = 1;
                sc->status = kStatusFallback;
            } else {
                sc->alpha = sc->rz / pq;
            }
            *ticket = 0u;
        }
    }
}

// The same over the upper-only FP32 layout: per row the lower blocks
// (transposes of their stored twins, ascending), then the stored blocks:
// the full layout's column order, so the same bits.  The stored blocks go
// through L2 normally, as the rows of the next two grid lines read them again.
// 6 CTAs per SM: 40 registers and no spill.  Measured per flexible-CG
// iteration at 400x400 (one box): 8 or 7 CTAs (32 registers, 40 B spilled)
// 90.5-90.8 us, 6 CTAs 86.0 us, 5 CTAs 87.7 us, 4 CTAs 90.0 us.
__global__ void __launch_bounds__(256, 6) k_fcg_spmv_sym(int32_t n, const int64_t *__restrict__ slice_base,
                                                      const int32_t *__restrict__ rowlen,
                                                      const uint8_t *__restrict__ pat_id,
                                                      const int32_t *__restrict__ pat_off,
                                                      const uint8_t *__restrict__ tpat_id,
                                                      const int2 *__restrict__ tpat,
                                                      const int32_t *__restrict__ tpat_len,
                                                      const float4 *__restrict__ K, const uint8_t *__restrict__ fixed,
                                                      const float2 *__restrict__ z, const float2 *__restrict__ p_old,
                                                      float2 *__restrict__ p_new, float2 *__restrict__ q, float *part,
                                                      int64_t n_part, unsigned *ticket, CGScalarsT<float> *sc)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    int64_t base = 0;
    int len = 0, pb = 0, tl = 0, tb = 0;
    if (i < n) {
        base = sell_row0<true>(__ldg(&slice_base[i >> 5]), i & 31);
        len = __ldg(&rowlen[i]);
        pb = (int)__ldg(&pat_id[i]) * kPatLen;
        const int tp = __ldg(&tpat_id[i]);
        tl = __ldg(&tpat_len[tp]);
        tb = tp * kPatLen;
    }
    pdl_wait();
    pdl_launch_dependents();
    if (*reinterpret_cast<volatile int *>(&sc->done)) return;
    const float beta = *reinterpret_cast<volatile float *>(&sc->beta);
    float v[1] = {0.f};
    if (i < n) {
        const uint64_t keep = l2_policy_keep();
        float y0 = 0.f, y1 = 0.f;
#pragma unroll 2
        for (int k = 0; k < tl; k++) {
            const int2 e = __ldg(&tpat[tb + k]);
            const int32_t c = i + e.x;
            const float4 a = transpose4(__ldcg(&K[sym_twin_slot(slice_base, c, e.y)]));
            const float2 zz = ld_keep(&z[c], keep), pp = ld_keep(&p_old[c], keep);
            const float px = fmaf(beta, pp.x, zz.x), py = fmaf(beta, pp.y, zz.y);
            y0 = fmaf(a.y, py, fmaf(a.x, px, y0));
            y1 = fmaf(a.w, py, fmaf(a.z, px, y1));
        }
#pragma unroll 4
        for (int k = 0; k < len; k++) {
            const int32_t c = i + __ldg(&pat_off[pb + k]);
            const float4 a = __ldcg(&K[base + sell_koff<true>(k)]);
            const float2 zz = ld_keep(&z[c], keep), pp = ld_keep(&p_old[c], keep);
            const float px = fmaf(beta, pp.x, zz.x), py = fmaf(beta, pp.y, zz.y);
            y0 = fmaf(a.y, py, fmaf(a.x, px, y0));
            y1 = fmaf(a.w, py, fmaf(a.z, px, y1));
        }
        if (fixed[2 * (int64_t)i]) y0 = 0.f;
        if (fixed[2 * (int64_t)i + 1]) y1 = 0.f;
        q[i] = make_float2(y0, y1);
        const float2 zi = z[i], pi = p_old[i];
        const float2 pn = make_float2(fmaf(beta, pi.x, zi.x), fmaf(beta, pi.y, zi.y));
        p_new[i] = pn;
        v[0] = fmaf(pn.y, y1, pn.x * y0);
    }
    if (fcg_partials<1>(v, part, n_part, ticket)) {
        float o[1];
        fcg_final<1>(part, n_part, o);
        if (threadIdx.x == 0) {
            const float pq = o[0];
            sc->pq = pq;
            if (!(pq > 0.f)) {
                sc->done = 1;
                sc->status = kStatusFallback;
            } else {
                sc->alpha = sc->rz / pq;
            }
            *ticket = 0u;
        }
    }
}

// x += alpha p, r_new = r_old - alpha q (the owner stores it, the factor
// pass forms it for its neighbours), y = G (sigma * r_new); partials of
// r_new.r_new; last CTA: convergence, stagnation and iteration limit
__global__ void __launch_bounds__(256, 8) k_fcg_update_first(int32_t n, GridInfo G, const uint2 *__restrict__ Gm,
                                                          const float2 *__restrict__ dinv,
                                                          const float2 *__restrict__ p, const float2 *__restrict__ q,
                                                          float2 *__restrict__ x, const float2 *__restrict__ r_old,
                                                          float2 *__restrict__ r_new, float2 *__restrict__ y,
                                                          float *part, int64_t n_part, unsigned *ticket,
                                                          CGScalarsT<float> *sc, int stall_window)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    // x and r_old (not written by the SpMV) before the wait; p, q, alpha and
    // the flag after it
    float2 xx = make_float2(0.f, 0.f), ro[NTRI];
    int32_t jn[NTRI];
    if (i < n) {
        xx = x[i];
#pragma unroll
        for (int k = 0; k < NTRI; k++) {
            jn[k] = patch_nbr(i, k, G);
            if (jn[k] >= 0) ro[k] = __ldg(&r_old[jn[k]]);
        }
    }
    pdl_wait();
    pdl_launch_dependents();
    if (*reinterpret_cast<volatile int *>(&sc->done)) return;
    const float alpha = *reinterpret_cast<volatile float *>(&sc->alpha);
    float v[1] = {0.f};
    if (i < n) {
        const float2 pp = p[i];
        xx.x = fmaf(alpha, pp.x, xx.x);
        xx.y = fmaf(alpha, pp.y, xx.y);
        x[i] = xx;
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < NTRI; k++) {
            if (jn[k] < 0) continue;
            const float2 qq = __ldg(&q[jn[k]]);
            const float2 rn = make_float2(fmaf(-alpha, qq.x, ro[k].x), fmaf(-alpha, qq.y, ro[k].y));
            if (k == 4) {
                r_new[i] = rn;
                v[0] = fmaf(rn.y, rn.y, rn.x * rn.x);
            }
            const float4 m = load_g(Gm, (int64_t)k * n + i);
            const float2 sg = sqrt2(__ldg(&dinv[jn[k]]));
            const float vx = sg.x * rn.x, vy = sg.y * rn.y;
            acc.x = fmaf(m.x, vx, fmaf(m.y, vy, acc.x));
            acc.y = fmaf(m.z, vx, fmaf(m.w, vy, acc.y));
        }
        y[i] = acc;
    }
    if (fcg_partials<1>(v, part, n_part, ticket)) {
        float o[1];
        fcg_final<1>(part, n_part, o);
        if (threadIdx.x == 0) {
            const float rr = o[0];
            sc->rr = rr;
            sc->iters += 1;
            if (rr < 0.98f * sc->rr_best) {
                sc->rr_best = rr;
                sc->it_best = sc->iters;
            }
            if (rr <= sc->thr) {
                sc->done = 1;
            } else if (!(rr == rr) || sc->iters - sc->it_best > max(stall_window, sc->it_best)) {
                sc->done = 1;
                sc->status = kStatusFallback;
            } else if (sc->iters >= sc->max_it) {
                sc->done = 1;
                sc->status = IPFEM_NONCONVERGED;
            }
            *ticket = 0u;
        }
    }
}

// ------------------------------------------------------------- training
// y = K x on an FP32 SELL tangent (Dirichlet rows 0), no reductions
template <bool PAT>
__global__ void __launch_bounds__(256) k_spmv32(int32_t n, const int64_t *__restrict__ slice_base,
                                                const int32_t *__restrict__ rowlen,
                                                const int32_t *__restrict__ sell_node,
                                                const int32_t *__restrict__ scol, const uint8_t *__restrict__ pat_id,
                                                const int32_t *__restrict__ pat_off, const float4 *__restrict__ K,
                                                const uint8_t *__restrict__ fixed, const float2 *__restrict__ x,
                                                float2 *__restrict__ y)
{
    const int32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int32_t i = sell_node[t];
    const int64_t base = sell_row0<true>(slice_base[t >> 5], t & 31);
    const int len = rowlen[t];
    const int pb = PAT ? (int)__ldg(&pat_id[t]) * kPatLen : 0;
    const uint64_t keep = l2_policy_keep();
    float y0 = 0.f, y1 = 0.f;
#pragma unroll 4
    for (int k = 0; k < len; k++) {
        const int64_t s = base + sell_koff<true>(k);
        const float4 a = __ldcs(&K[s]);
        const float2 v = ld_keep(&x[PAT ? i + __ldg(&pat_off[pb + k]) : __ldg(&scol[s])], keep);
        y0 = fmaf(a.x, v.x, fmaf(a.y, v.y, y0));
        y1 = fmaf(a.z, v.x, fmaf(a.w, v.y, y1));
    }
    if (fixed[2 * (int64_t)i]) y0 = 0.f;
    if (fixed[2 * (int64_t)i + 1]) y1 = 0.f;
    y[i] = make_float2(y0, y1);
}

// the same over the upper-only layout: the lower blocks (transposes of their
// stored twins, ascending) first, then the stored ones: the full layout's
// column order, so the same bits
__global__ void __launch_bounds__(256) k_spmv32_sym(int32_t n, const int64_t *__restrict__ slice_base,
                                                    const int32_t *__restrict__ rowlen,
                                                    const uint8_t *__restrict__ pat_id,
                                                    const int32_t *__restrict__ pat_off,
                                                    const uint8_t *__restrict__ tpat_id, const int2 *__restrict__ tpat,
                                                    const int32_t *__restrict__ tpat_len, const float4 *__restrict__ K,
                                                    const uint8_t *__restrict__ fixed, const float2 *__restrict__ x,
                                                    float2 *__restrict__ y)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t base = sell_row0<true>(slice_base[i >> 5], i & 31);
    const int len = rowlen[i];
    const int pb = (int)__ldg(&pat_id[i]) * kPatLen;
    const int tp = __ldg(&tpat_id[i]);
    const int tl = __ldg(&tpat_len[tp]), tb = tp * kPatLen;
    const uint64_t keep = l2_policy_keep();
    float y0 = 0.f, y1 = 0.f;
#pragma unroll 4
    for (int k = 0; k < tl; k++) {
        const int2 e = __ldg(&tpat[tb + k]);
        const int32_t j = i + e.x;
        const float4 a = transpose4(__ldcg(&K[sym_twin_slot(slice_base, j, e.y)]));
        const float2 v = ld_keep(&x[j], keep);
        y0 = fmaf(a.x, v.x, fmaf(a.y, v.y, y0));
        y1 = fmaf(a.z, v.x, fmaf(a.w, v.y, y1));
    }
#pragma unroll 4
    for (int k = 0; k < len; k++) {
        const float4 a = __ldcg(&K[base + sell_koff<true>(k)]);
        const float2 v = ld_keep(&x[i + __ldg(&pat_off[pb + k])], keep);
        y0 = fmaf(a.x, v.x, fmaf(a.y, v.y, y0));
        y1 = fmaf(a.z, v.x, fmaf(a.w, v.y, y1));
    }
    if (fixed[2 * (int64_t)i]) y0 = 0.f;
    if (fixed[2 * (int64_t)i + 1]) y1 = 0.f;
    y[i] = make_float2(y0, y1);
}

// res = ae - az; CTA partials of ae.ae and res.res into part[2][gridDim.x]
__global__ void __launch_bounds__(256) k_res_part(int64_t neq, const float *__restrict__ ae,
                                                  const float *__restrict__ az, float *__restrict__ res,
                                                  float *__restrict__ part)
{
    __shared__ float ws[2][8];
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    float a = 0.f, b = 0.f;
    if (i < neq) {
        const float e = ae[i], d = e - az[i];
        res[i] = d;
        a = e * e;
        b = d * d;
    }
    a = wsum(a);
    b = wsum(b);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        ws[0][w] = a;
        ws[1][w] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float sa = 0.f, sb = 0.f;
        for (int k = 0; k < 8; k++) {
            sa += ws[0][k];
            sb += ws[1][k];
        }
        part[blockIdx.x] = sa;
        part[gridDim.x + blockIdx.x] = sb;
    }
}

// scal[0] = ae.ae, scal[1] = res.res; loss += res.res / ae.ae * w
__global__ void __launch_bounds__(256) k_res_final(int n_part, const float *__restrict__ part, float *__restrict__ scal,
                                                   float *__restrict__ loss, float w)
{
    __shared__ float ws[2][8];
    float a = 0.f, b = 0.f;
    for (int i = threadIdx.x; i < n_part; i += blockDim.x) {
        a += part[i];
        b += part[n_part + i];
    }
    a = wsum(a);
    b = wsum(b);
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    if (lane == 0) {
        ws[0][wp] = a;
        ws[1][wp] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float sa = 0.f, sb = 0.f;
        for (int k = 0; k < 8; k++) {
            sa += ws[0][k];
            sb += ws[1][k];
        }
        scal[0] = sa;
        scal[1] = sb;
        if (sa > 0.f) *loss += sb / sa * w;
    }
}

// Pair term of dL/dG for z = sigma G^T G sigma r: with rh = sigma*r,
// u = sigma*g (g = K (ae - az)), y = G rh, v = G u and c = -2 w / ae.ae,
// dG_ik[p][q] += c (y_i[p] u_j[q] + v_i[p] rh_j[q]),  j = nbr(i, k)
__global__ void __launch_bounds__(256) k_tri_grad_pairs(int32_t n, GridInfo G, const float2 *__restrict__ dinv,
                                                        const float2 *__restrict__ r, const float2 *__restrict__ g,
                                                        const float2 *__restrict__ y, const float2 *__restrict__ v,
                                                        const float *__restrict__ scal, float w,
                                                        float *__restrict__ dG)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !(scal[0] > 0.f)) return;
    const float c = -2.f * w / scal[0];
    const float2 yi = y[i], vi = v[i];
    float *o = dG + (int64_t)i * NOUT;
#pragma unroll
    for (int k = 0; k < NTRI; k++) {
        const int32_t j = patch_nbr(i, k, G);
        if (j < 0) continue;
        const float2 sj = sqrt2(dinv[j]);
        const float2 rj = make_float2(sj.x * r[j].x, sj.y * r[j].y);
        const float2 uj = make_float2(sj.x * g[j].x, sj.y * g[j].y);
        o[4 * k + 0] += c * (yi.x * uj.x + vi.x * rj.x);
        o[4 * k + 1] += c * (yi.x * uj.y + vi.x * rj.y);
        o[4 * k + 2] += c * (yi.y * uj.x + vi.y * rj.x);
        o[4 * k + 3] += c * (yi.y * uj.y + vi.y * rj.y);
    }
}

// Kaporin term, per node i with patch nodes j_k = nbr(i, k), k = 0..4:
// H_ik[p][q] = sum_l sum_t Ahat[(j_k, q), (j_l, t)] G_il[p][t] with
// Ahat = sigma K sigma (pslot[5k + l][i] = slot of block (j_k, j_l) or -1);
// CTA partials of sum G.H (= the node's share of tr(G Ahat G^T)) and of the
// log-diagonal sum f0 O[16] + f1 O[18] into part[2][gridDim.x]
__global__ void __launch_bounds__(256) k_kap_H(int32_t n, GridInfo G, const float4 *__restrict__ Gm,
                                               const float4 *__restrict__ K, const int32_t *__restrict__ pslot,
                                               const float2 *__restrict__ dinv, const float *__restrict__ O,
                                               float *__restrict__ H, float *__restrict__ part)
{
    __shared__ float ws[2][8];
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float tr = 0.f, ld = 0.f;
    if (i < n) {
        float4 gl[NTRI];
        float2 sl[NTRI];
#pragma unroll
        for (int l = 0; l < NTRI; l++) {
            gl[l] = Gm[(int64_t)l * n + i];
            const int32_t j = patch_nbr(i, l, G);
            sl[l] = j >= 0 ? sqrt2(dinv[j]) : make_float2(0.f, 0.f);
        }
        float *h = H + (int64_t)i * NOUT;
#pragma unroll
        for (int k = 0; k < NTRI; k++) {
            float h00 = 0.f, h01 = 0.f, h10 = 0.f, h11 = 0.f;
#pragma unroll
            for (int l = 0; l < NTRI; l++) {
                const int32_t s = pslot[(int64_t)(NTRI * k + l) * n + i];
                if (s == -1) continue;
                const float4 kb = tangent_block(K, s);
                // Ahat[q][t] for q (row, node j_k), t (column, node j_l)
                const float a00 = sl[k].x * kb.x * sl[l].x, a01 = sl[k].x * kb.y * sl[l].y;
                const float a10 = sl[k].y * kb.z * sl[l].x, a11 = sl[k].y * kb.w * sl[l].y;
                // H[p][q] += sum_t G_l[p][t] Ahat[q][t]
                h00 += gl[l].x * a00 + gl[l].y * a01;
                h01 += gl[l].x * a10 + gl[l].y * a11;
                h10 += gl[l].z * a00 + gl[l].w * a01;
                h11 += gl[l].z * a10 + gl[l].w * a11;
            }
            h[4 * k + 0] = h00;
            h[4 * k + 1] = h01;
            h[4 * k + 2] = h10;
            h[4 * k + 3] = h11;
            tr += gl[k].x * h00 + gl[k].y * h01 + gl[k].z * h10 + gl[k].w * h11;
        }
        const float2 f = free2(dinv[i]);
        ld = f.x * O[(int64_t)i * NOUT + 16] + f.y * O[(int64_t)i * NOUT + 18];
    }
    tr = wsum(tr);
    ld = wsum(ld);
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    if (lane == 0) {
        ws[0][wp] = tr;
        ws[1][wp] = ld;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float a = 0.f, b = 0.f;
        for (int k = 0; k < 8; k++) {
            a += ws[0][k];
            b += ws[1][k];
        }
        part[blockIdx.x] = a;
        part[gridDim.x + blockIdx.x] = b;
    }
}

// scal[2] = T = tr(G Ahat G^T), scal[3] = sum of the log-diagonal;
// loss += wk (log(T / nf) - 2 LD / nf)
__global__ void __launch_bounds__(256) k_kap_final(int n_part, const float *__restrict__ part,
                                                   float *__restrict__ scal, float *__restrict__ loss, float wk,
                                                   float nf)
{
    __shared__ float ws[2][8];
    float a = 0.f, b = 0.f;
    for (int i = threadIdx.x; i < n_part; i += blockDim.x) {
        a += part[i];
        b += part[n_part + i];
    }
    a = wsum(a);
    b = wsum(b);
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    if (lane == 0) {
        ws[0][wp] = a;
        ws[1][wp] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float sa = 0.f, sb = 0.f;
        for (int k = 0; k < 8; k++) {
            sa += ws[0][k];
            sb += ws[1][k];
        }
        scal[2] = sa;
        scal[3] = sb;
        *loss += wk * (logf(sa / nf) - 2.f * sb / nf);
    }
}

// dL/dO from dG (pair term) + wk (2/T) H (Kaporin trace) through G(O), plus
// the log-determinant term -2 wk / nf on O[16], O[18] of free dofs
__global__ void __launch_bounds__(256) k_tri_dO(int32_t n, GridInfo G, const float *__restrict__ O,
                                                const float2 *__restrict__ dinv, const float *__restrict__ dG,
                                                const float *__restrict__ H, const float *__restrict__ scal, float wk,
                                                float nf, float *__restrict__ dO)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float ck = scal[2] > 0.f ? 2.f * wk / scal[2] : 0.f;
    const float2 fi = free2(dinv[i]);
    const float *gi = dG + (int64_t)i * NOUT, *hi = H + (int64_t)i * NOUT, *oi = O + (int64_t)i * NOUT;
    float *d = dO + (int64_t)i * NOUT;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int32_t j = patch_nbr(i, k, G);
        const float2 fj = j >= 0 ? free2(dinv[j]) : make_float2(0.f, 0.f);
        d[4 * k + 0] = (gi[4 * k + 0] + ck * hi[4 * k + 0]) * fi.x * fj.x;
        d[4 * k + 1] = (gi[4 * k + 1] + ck * hi[4 * k + 1]) * fi.x * fj.y;
        d[4 * k + 2] = (gi[4 * k + 2] + ck * hi[4 * k + 2]) * fi.y * fj.x;
        d[4 * k + 3] = (gi[4 * k + 3] + ck * hi[4 * k + 3]) * fi.y * fj.y;
    }
    const bool in16 = fabsf(oi[16]) < 30.f, in18 = fabsf(oi[18]) < 30.f;
    d[16] = in16 ? ((gi[16] + ck * hi[16]) * expf(oi[16]) - 2.f * wk / nf) * fi.x : 0.f;
    d[17] = (gi[18] + ck * hi[18]) * fi.y * fi.x;
    d[18] = in18 ? ((gi[19] + ck * hi[19]) * expf(oi[18]) - 2.f * wk / nf) * fi.y : 0.f;
    d[19] = 0.f;
}

// ---------------------------------------------------------------- host side

// BF16 copies of W1, W2, W3 in the (n, k) layout of the tensor-core B operand
__global__ void k_pack_w(const float *__restrict__ P, __nv_bfloat16 *__restrict__ w1t, __nv_bfloat16 *__restrict__ w2t,
                         __nv_bfloat16 *__restrict__ w3t)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 128 * 32) {
        const int n = i / 32, k = i % 32;
        w1t[i] = __float2bfloat16_rn(P[kOffW1 + k * 128 + n]);
    }
    if (i < 128 * 128) {
        const int n = i / 128, k = i % 128;
        w2t[i] = __float2bfloat16_rn(P[kOffW2 + k * 128 + n]);
    }
    if (i < NOUTP * 128) {
        const int n = i / 128, k = i % 128;
        w3t[i] = __float2bfloat16_rn(n < NOUT ? P[kOffW3 + k * NOUT + n] : 0.f);
    }
}

void mlp_pack_weights(ipfem_ctx *c)
{
    MlpBuffers &m = c->mlp;
    k_pack_w<<<64, 256, 0, c->stream>>>(m.params, static_cast<__nv_bfloat16 *>(m.w1t),
                                        static_cast<__nv_bfloat16 *>(m.w2t), static_cast<__nv_bfloat16 *>(m.w3t));
    m.op_valid = false;
}

// opt-in to the shared memory of the fused network kernel (once, outside any capture)
cudaError_t mlp_configure()
{
    return net_tc_configure();
}

void launch_patch_net(ipfem_ctx *c, int64_t rows, const float *d_X, float *d_O)
{
    launch_patch_net_tc(c, rows, d_X, d_O);
}

void launch_patch_features(ipfem_ctx *c, float *d_X)
{
    const int32_t n = c->s.n_nodes;
    GridInfo G{c->mlp.gr, c->mlp.gt};
    k_patch_features<<<(n + 255) / 256, 256, 0, c->stream>>>(n, G, reinterpret_cast<const float4 *>(fp32_values(c)),
                                                             use_sym32(c) ? c->mlp.slot_s : c->mlp.slot,
                                                             reinterpret_cast<const float2 *>(c->mx.dinv), d_X);
}

// features -> network -> triangular factor, for the current FP32 tangent
void launch_patch_operator(ipfem_ctx *c)
{
    MlpBuffers &m = c->mlp;
    const int32_t n = c->s.n_nodes;
    GridInfo G{m.gr, m.gt};
    launch_patch_features(c, m.X);
    launch_patch_net(c, n, m.X, m.O);
    k_tri_build<<<(n + 255) / 256, 256, 0, c->stream>>>(n, G, m.O, reinterpret_cast<const float2 *>(c->mx.dinv),
                                                        reinterpret_cast<float4 *>(m.M),
                                                        reinterpret_cast<uint2 *>(m.Gh));
    c->launches += 3;
    m.op_valid = true;
}

// FCG gives up (and the caller falls back to Jacobi-PCG) when |r|^2 has not
// dropped by 2 % for max(stall window, iterations to the best |r|^2 so far)
// iterations.  CG minimises the energy norm of the error, not |r|, and its
// residual can stay near its initial value for a number of iterations that
// grows with the grid width, so the window is max(2000, 2 sqrt(neq)).  M is
// SPD, so this only guards against a network far outside its training data.
static int stall_window(const ipfem_ctx *c)
{
    return (int)std::max(2000.0, 2.0 * std::sqrt((double)c->s.neq));
}

static unsigned fcg_grid(const ipfem_ctx *c)
{
    return (unsigned)((c->s.n_nodes + 255) / 256);
}

// z = M r for r = R[par] (r_old = R[1 - par]), the two factor passes
static void launch_precond(ipfem_ctx *c, int par)
{
    GridInfo G{c->mlp.gr, c->mlp.gt};
    MixedBuffers &m = c->mx;
    float *R[2] = {m.r, c->mlp.r_old};
    // the precond partials use the FP64 partial array (as 2 x n_red floats)
    float *part = reinterpret_cast<float *>(c->d_part);
    const uint2 *Gh = reinterpret_cast<const uint2 *>(c->mlp.Gh);
    const float2 *d2 = reinterpret_cast<const float2 *>(m.dinv);
    float2 *y = reinterpret_cast<float2 *>(c->mlp.y);
    k_tri_first<<<fcg_grid(c), 256, 0, c->stream>>>(c->s.n_nodes, G, Gh, d2, reinterpret_cast<const float2 *>(R[par]),
                                                    y, m.sc);
    k_tri_precond<<<fcg_grid(c), 256, 0, c->stream>>>(c->s.n_nodes, G, Gh, d2, y, R[par], R[1 - par], m.z, part,
                                                      (int64_t)fcg_grid(c), c->d_counters + 7, m.sc);
}

// r = R[0] = b*scale, x = 0, P[0] = 0, R[1] = 0; z = M r and beta = 0
void launch_fcg_init(ipfem_ctx *c, const double *d_b, double scale, float rtol, int max_it)
{
    MixedBuffers &m = c->mx;
    k_fcg_init<<<fcg_grid(c), 256, 0, c->stream>>>(c->s.n_nodes, d_b, scale, m.x, m.r, m.p, c->mlp.r_old, m.part,
                                                   (int64_t)fcg_grid(c), c->d_counters + 4, m.sc, rtol, max_it);
    launch_precond(c, 0);
}

// iteration k (par = k % 2): P[par] -> P[1-par] in the SpMV, R[par] -> R[1-par]
// in the update, z from R[1-par]
void launch_fcg_iteration(ipfem_ctx *c, int par)
{
    MixedBuffers &m = c->mx;
    MlpBuffers &l = c->mlp;
    const SellDev &L = fp32_layout(c);
    GridInfo G{l.gr, l.gt};
    const int32_t n = c->s.n_nodes;
    float2 *P[2] = {reinterpret_cast<float2 *>(m.p), reinterpret_cast<float2 *>(l.p2)};
    float2 *R[2] = {reinterpret_cast<float2 *>(m.r), reinterpret_cast<float2 *>(l.r_old)};
    const float2 *d2 = reinterpret_cast<const float2 *>(m.dinv);
    float *part = m.part;
    if (L.sym)
        launch_pdl(k_fcg_spmv_sym, fcg_grid(c), 256, c->stream, n, (const int64_t *)L.slice_base,
                   (const int32_t *)L.rowlen, (const uint8_t *)L.pat_id, (const int32_t *)L.pat_off,
                   (const uint8_t *)L.tpat_id, (const int2 *)L.tpat, (const int32_t *)L.tpat_len,
                   reinterpret_cast<const float4 *>(fp32_values(c)), (const uint8_t *)c->d_fixed,
                   reinterpret_cast<const float2 *>(m.z), (const float2 *)P[par], P[1 - par],
                   reinterpret_cast<float2 *>(m.q), part, (int64_t)fcg_grid(c), c->d_counters + 5, m.sc);
    else
        launch_pdl(use_row_stencils(c, L) ? k_fcg_spmv<true> : k_fcg_spmv<false>, fcg_grid(c), 256, c->stream, n,
                   (const int64_t *)L.slice_base, (const int32_t *)L.rowlen, (const int32_t *)L.sell_col,
                   (const uint8_t *)L.pat_id, (const int32_t *)L.pat_off, reinterpret_cast<const float4 *>(m.K),
                   (const uint8_t *)c->d_fixed, reinterpret_cast<const float2 *>(m.z), (const float2 *)P[par],
                   P[1 - par], reinterpret_cast<float2 *>(m.q), part, (int64_t)fcg_grid(c), c->d_counters + 5, m.sc);
    launch_pdl(k_fcg_update_first, fcg_grid(c), 256, c->stream, n, G, reinterpret_cast<const uint2 *>(l.Gh), d2,
               (const float2 *)P[1 - par], reinterpret_cast<const float2 *>(m.q), reinterpret_cast<float2 *>(m.x),
               (const float2 *)R[par], R[1 - par], reinterpret_cast<float2 *>(l.y), part, (int64_t)fcg_grid(c),
               c->d_counters + 6, m.sc, stall_window(c));
    float *part2 = reinterpret_cast<float *>(c->d_part);
    launch_pdl(k_tri_precond, fcg_grid(c), 256, c->stream, n, G, reinterpret_cast<const uint2 *>(l.Gh), d2,
               reinterpret_cast<const float2 *>(l.y), reinterpret_cast<const float *>(R[1 - par]),
               reinterpret_cast<const float *>(R[par]), m.z, part2, (int64_t)fcg_grid(c), c->d_counters + 7, m.sc);
}

// ------------------------------------------------------------ training pass
// The weight-gradient GEMMs split their K (= rows) into at most kMaxSplits
// ranges of a multiple of 32 rows: 4 CTAs on each of 152 SMs, one wave.
constexpr int kMaxSplits = 608;

static int split_rows(int64_t rows)
{
    const int64_t per = (rows + kMaxSplits - 1) / kMaxSplits;
    return (int)std::max<int64_t>(32, (per + 31) / 32 * 32);
}

// C[M][N] = A^T B over K = rows (both row-major with rows as the K index),
// split K; colsum[N] = the column sums of B (1^T B) from the same pass
static void gemm_tn_split(ipfem_ctx *c, int M, int N, int64_t rows, const float *A, int lda, const float *B, int ldb,
                          float *C, float *colsum)
{
    MlpBuffers &m = c->mlp;
    const int kchunk = split_rows(rows);
    const int splits = (int)((rows + kchunk - 1) / kchunk);
    float *cpart = m.part + (size_t)kMaxSplits * 128 * 128;
    launch_gemm_tc(c, M, N, (int)rows, A, lda, 1, B, ldb, 0, m.part, N, kchunk, splits, cpart);
    const int64_t n = (int64_t)M * N;
    k_sum_splits<<<(unsigned)((n + 31) / 32), 256, 0, c->stream>>>(n, splits, m.part, C);
    k_sum_splits<<<(unsigned)((N + 31) / 32), 256, 0, c->stream>>>(N, splits, cpart, colsum);
}

// floats of mlp.part: the split-K partials of a 128 x 128 weight gradient and
// of its column sums
size_t patch_part_floats(int64_t)
{
    return (size_t)kMaxSplits * (128 * 128 + 128);
}

// Gradient of
//   L = wk (log(tr(G Ahat G^T) / nf) - (2/nf) log det G)
//     + wp (1/P) sum_p |K e_p - K M r_p|^2 / |K e_p|^2   (M = sigma G^T G sigma)
// with respect to the parameters (into mlp.grads) and L (into mlp.loss), for
// P >= 0 pairs of FP32 device vectors r_p = d_r + p*neq, e_p = d_e + p*neq on
// this tangent; nf = number of free dofs.
void patch_learn_grad(ipfem_ctx *c, const float *d_r, const float *d_e, int P, float wk, float wp)
{
    MlpBuffers &m = c->mlp;
    MixedBuffers &x = c->mx;
    const Setup &s = c->s;
    const int32_t n = s.n_nodes;
    const int64_t neq = s.neq;
    cudaStream_t st = c->stream;
    GridInfo G{m.gr, m.gt};
    const unsigned gn = (unsigned)((n + 255) / 256);
    const unsigned ge = (unsigned)((neq + 255) / 256);
    const float2 *d2 = reinterpret_cast<const float2 *>(x.dinv);
    float4 *Gm = reinterpret_cast<float4 *>(m.M);
    // forward through the fused network kernel, which also writes the hidden layers for the backward
    launch_patch_features(c, m.X);
    launch_patch_net_tc(c, n, m.X, m.O, m.H1, m.H2);
    k_tri_build<<<gn, 256, 0, st>>>(n, G, m.O, d2, Gm, nullptr);
    m.op_valid = false;
    cudaMemsetAsync(m.dN, 0, (size_t)n * NOUT * sizeof(float), st);
    cudaMemsetAsync(m.loss, 0, sizeof(float), st);
    // pair term
    float *z = m.vec, *ae = m.vec + neq, *az = m.vec + 2 * neq, *res = m.vec + 3 * neq, *g = m.vec + 4 * neq;
    float *y = m.vec + 5 * neq, *v = m.vec + 6 * neq;
    const SellDev &L = fp32_layout(c);
    const float4 *K4 = reinterpret_cast<const float4 *>(fp32_values(c));
    const float w = P > 0 ? wp / (float)P : 0.f;
    auto spmv32 = [&](const float2 *xin, float2 *yout) {
        if (L.sym)
            k_spmv32_sym<<<gn, 256, 0, st>>>(n, L.slice_base, L.rowlen, L.pat_id, L.pat_off, L.tpat_id, L.tpat,
                                              L.tpat_len, K4, c->d_fixed, xin, yout);
        else
            (use_row_stencils(c, L) ? k_spmv32<true> : k_spmv32<false>)<<<gn, 256, 0, st>>>(
                n, L.slice_base, L.rowlen, L.sell_node, L.sell_col, L.pat_id, L.pat_off, K4, c->d_fixed, xin, yout);
    };
    for (int p = 0; p < P && wp > 0.f; p++) {
        const float2 *r2 = reinterpret_cast<const float2 *>(d_r + (size_t)p * neq);
        const float2 *e2 = reinterpret_cast<const float2 *>(d_e + (size_t)p * neq);
        k_tri_first<<<gn, 256, 0, st>>>(n, G, Gm, d2, r2, reinterpret_cast<float2 *>(y), nullptr);
        k_tri_second<<<gn, 256, 0, st>>>(n, G, Gm, d2, reinterpret_cast<const float2 *>(y),
                                         reinterpret_cast<float2 *>(z));
        spmv32(e2, reinterpret_cast<float2 *>(ae));
        spmv32(reinterpret_cast<const float2 *>(z), reinterpret_cast<float2 *>(az));
        k_res_part<<<ge, 256, 0, st>>>(neq, ae, az, res, m.part);
        k_res_final<<<1, 256, 0, st>>>((int)ge, m.part, m.scal, m.loss, w);
        spmv32(reinterpret_cast<const float2 *>(res), reinterpret_cast<float2 *>(g));
        k_tri_first<<<gn, 256, 0, st>>>(n, G, Gm, d2, reinterpret_cast<const float2 *>(g),
                                        reinterpret_cast<float2 *>(v), nullptr);
        k_tri_grad_pairs<<<gn, 256, 0, st>>>(n, G, d2, r2, reinterpret_cast<const float2 *>(g),
                                             reinterpret_cast<const float2 *>(y), reinterpret_cast<const float2 *>(v),
                                             m.scal, w, m.dN);
    }
    // Kaporin term (H in the dH1 buffer, free before the backward)
    float *H = m.dH1;
    k_kap_H<<<gn, 256, 0, st>>>(n, G, Gm, K4, use_sym32(c) ? m.pslot_s : m.pslot, d2, m.O, H, m.part);
    k_kap_final<<<1, 256, 0, st>>>((int)gn, m.part, m.scal, m.loss, wk, m.nf);
    float *dO = m.dH2;                      // [n][20], free until dH2 is formed
    k_tri_dO<<<gn, 256, 0, st>>>(n, G, m.O, d2, m.dN, H, m.scal, wk, m.nf, dO);
    cudaMemcpyAsync(m.dN, dO, (size_t)n * NOUT * sizeof(float), cudaMemcpyDeviceToDevice, st);
    // backward
    float *gr = m.grads;
    gemm_tn_split(c, 128, NOUT, n, m.H2, 128, m.dN, NOUT, gr + kOffW3, gr + kOffB3);  // dW3 = H2^T dO
    launch_patch_net_bwd_tc(c, n, m.dN, m.H1, m.H2, m.dH2, m.dH1);                    // dH2, dH1
    gemm_tn_split(c, 128, 128, n, m.H1, 128, m.dH2, 128, gr + kOffW2, gr + kOffB2);  // dW2 = H1^T dH2
    gemm_tn_split(c, 32, 128, n, m.X, 32, m.dH1, 128, gr + kOffW1, gr + kOffB1);      // dW1 = X^T dH1
    c->launches += 3 + 9 * (uint64_t)(wp > 0.f ? P : 0) + 3 + 10;
}

// one Adam step on the parameters with the gradient in mlp.grads
void mlp_adam_step(ipfem_ctx *c, float lr)
{
    MlpBuffers &m = c->mlp;
    m.adam_t += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)m.adam_t), c2 = 1.f - powf(b2, (float)m.adam_t);
    k_adam<<<(kMlpParams + 255) / 256, 256, 0, c->stream>>>(kMlpParams, m.params, m.grads, m.m, m.v, lr, b1, b2,
                                                             1e-8f, c1, c2);
    mlp_pack_weights(c);
    c->launches += 2;
}

}  // namespace ipfem
