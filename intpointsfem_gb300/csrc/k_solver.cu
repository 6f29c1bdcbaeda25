// Jacobi-preconditioned CG on the nodal 2x2 block tangent, FP64.
//
// The reference assembles K into a symmetric CSR and solves with Pardiso
// (main.cpp:283-285); its only CG (TPZCudaCalls::SolveCG, TPZCudaCalls.cu:213-290)
// is unpreconditioned and unused.  Here the matrix is stored as 2x2 blocks in
// SELL-32 order (slice of 32 node rows, slot-major, lane-minor) so that a
// warp reads one slot of 32 rows as 1 KB of contiguous values.
//
// Every dot product follows one canonical reduction order (shared with the CPU
// oracle): per node fma(a0,b0,0) then fma(a1,b1,.), a 32-lane shuffle-down
// tree, a tree over the 8 warps of a 256-node CTA, and a last-CTA final pass
// (256 threads strided over the CTA partials, then the same trees).  With
// fma-ordered SpMV and vector updates, the whole solve is deterministic and
// equal to the oracle bit for bit.
//
// Scalars (alpha, beta, convergence) live in device memory, so an iteration
// is three kernels with no host round trip; the host replays a captured CUDA
// graph of several iterations and checks the `done` word between replays.
#include "ipfem_internal.h"
#include "ldhint.cuh"
#include "pdl.cuh"

namespace ipfem {

constexpr unsigned FULL = 0xffffffffu;


template <class T>
__device__ __forceinline__ T warp_tree(T v)
{
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v = v + __shfl_down_sync(FULL, v, off);
    return v;
}

// tree over the 8 warp sums in shared memory (4, 2, 1); valid in thread 0
template <class T>
__device__ __forceinline__ T tree8(const volatile T *w)
{
    T a[8];
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = w[k];
#pragma unroll
    for (int off = 4; off >= 1; off >>= 1)
#pragma unroll
        for (int l = 0; l < off; l++) a[l] = a[l] + a[l + off];
    return a[0];
}

// Level 0+1 of one 256-node window, evaluated by a single warp.  The pairing
// is exactly the shuffle-down tree above (node t = 32 w + l, l = l4..l0: pairs
// over l4, l3, l2, l1, l0) followed by tree8 over the warps (w2, w1, w0), so
// the sum is bit-identical to warp_tree + tree8; only its evaluation differs.
// The values are staged in shared memory at stage(t) = 34 (t >> 5) + (t & 31)
// (stride 34 keeps the gathers below free of bank conflicts for FP64).  Lane
// j = 16 l1 + 8 l0 + w of warp 0 loads the 8 values with its (l1, l0, w),
// adds over l4, l3, l2 in registers (7 adds, every lane useful) and over
// l1, l0, w2, w1, w0 by shuffles.  That is 12 warp-wide FP64 adds per value
// against 47 for the 8 shuffle trees plus tree8 — the FP64 pipe bounds the
// vector-update kernels on this part.
constexpr int kRedPad = 34;
constexpr int kRedStage = 8 * kRedPad;
__device__ __forceinline__ int red_stage(int t) { return (t >> 5) * kRedPad + (t & 31); }

template <class T>
__device__ __forceinline__ T tree256_warp(const T *s)
{
    const int lane = threadIdx.x & 31;
    const T *b = s + (lane & 7) * kRedPad + 2 * (lane >> 4) + ((lane >> 3) & 1);
    T x[8];
#pragma unroll
    for (int m = 0; m < 8; m++) x[m] = b[4 * m];
#pragma unroll
    for (int m = 0; m < 4; m++) x[m] = x[m] + x[m + 4];
    x[0] = x[0] + x[2];
    x[1] = x[1] + x[3];
    T u = x[0] + x[1];
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) u = u + __shfl_down_sync(FULL, u, off);
    return u;
}

// Per-CTA partial sums of values the caller has staged (s[k][red_stage(t)]
// for the node in slot t, zero for empty slots) and synchronised; written to
// part[k][blockIdx].  Returns true in every thread of the CTA that finished
// last (after a fence).  Value k is summed by warp (blockIdx + 2k) mod 4: a
// warp-wide FP64 add occupies its SM sub-partition's FP64 unit for many
// cycles, and warps w, w+4 of a CTA share a sub-partition, so rotating the
// summing warp over the CTAs resident on an SM (and giving the two values of
// one CTA different warps) spreads the trees over all four sub-partitions
// instead of stacking every resident CTA's tree on one.
template <class T, int NV>
__device__ __forceinline__ bool block_partials_staged(const T (*s)[kRedStage], T *part, int64_t n_red,
                                                      unsigned *ticket)
{
    static_assert(NV == 1 || NV == 2, "one or two values");
    __shared__ int s_last;
    __shared__ T s_res[NV];
    const int w = threadIdx.x >> 5;
    const int w0 = (int)(blockIdx.x & 3u);
    // one thread writes every partial, fences and takes the ticket
    if (NV == 1) {
        if (w == w0) {
            const T o = tree256_warp<T>(s[0]);
            if ((threadIdx.x & 31) == 0) {
                part[blockIdx.x] = o;
                __threadfence();
                const unsigned t = atomicAdd(ticket, 1u);
                s_last = (t == gridDim.x - 1);
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < NV; k++)
            if (w == ((w0 + 2 * k) & 3)) {
                const T o = tree256_warp<T>(s[k]);
                if ((threadIdx.x & 31) == 0) s_res[k] = o;
            }
        __syncthreads();
        if (threadIdx.x == 0) {
#pragma unroll
            for (int k = 0; k < NV; k++) part[k * n_red + blockIdx.x] = s_res[k];
            __threadfence();
            const unsigned t = atomicAdd(ticket, 1u);
            s_last = (t == gridDim.x - 1);
        }
    }
    __syncthreads();
    return s_last != 0;
}

// The same for one value per thread, thread t holding node slot t.
template <class T, int NV>
__device__ __forceinline__ bool block_partials(const T (&v)[NV], T *part, int64_t n_red, unsigned *ticket)
{
    __shared__ T s[NV][kRedStage];
#pragma unroll
    for (int k = 0; k < NV; k++) s[k][red_stage(threadIdx.x)] = v[k];
    __syncthreads();
    return block_partials_staged<T, NV>(s, part, n_red, ticket);
}

// Level 2, executed by all 256 threads of the last CTA; result valid in thread 0.
template <class T, int NV>
__device__ __forceinline__ void final_reduce(const T *part, int64_t n_red, T (&out)[NV])
{
    __shared__ T ws[NV][8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        // strided partials t, t+256, t+512, ... summed in that order; four loads
        // are issued before their adds so that the pass is not latency-serial
        const T *pk = part + k * n_red;
        T acc = T(0);
        int64_t i = threadIdx.x;
        for (; i + 3 * kRedBlock < n_red; i += 4 * kRedBlock) {
            const T v0 = __ldcg(&pk[i]), v1 = __ldcg(&pk[i + kRedBlock]);
            const T v2 = __ldcg(&pk[i + 2 * kRedBlock]), v3 = __ldcg(&pk[i + 3 * kRedBlock]);
            acc = acc + v0;
            acc = acc + v1;
            acc = acc + v2;
            acc = acc + v3;
        }
        for (; i < n_red; i += kRedBlock) acc = acc + __ldcg(&pk[i]);
        acc = warp_tree(acc);
        if (lane == 0) ws[k][w] = acc;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) out[k] = tree8<T>(ws[k]);
    }
}

template <class T> struct Vec2;
template <> struct Vec2<double> { typedef double2 type; };
template <> struct Vec2<float> { typedef float2 type; };

__device__ __forceinline__ double2 mk2(double a, double b) { return make_double2(a, b); }
__device__ __forceinline__ float2 mk2(float a, float b) { return make_float2(a, b); }

// 2x2 block s of a SELL matrix: FP64 as two 16-byte loads, FP32 as one;
// streamed (evict-first: each block is read once per SpMV)
__device__ __forceinline__ void load_block(const double *K, int64_t s, double &a, double &b, double &c, double &d)
{
    const double2 *Kv = reinterpret_cast<const double2 *>(K);
    const double2 u = __ldcs(&Kv[2 * s]), v = __ldcs(&Kv[2 * s + 1]);
    a = u.x; b = u.y; c = v.x; d = v.y;
}
__device__ __forceinline__ void load_block(const float *K, int64_t s, float &a, float &b, float &c, float &d)
{
    const float4 u = __ldcs(&reinterpret_cast<const float4 *>(K)[s]);
    a = u.x; b = u.y; c = u.z; d = u.w;
}

// z = M r at node i: Jacobi (minv = dinv[2 n]) or block Jacobi (minv = binv[4 n]:
// z0 = fma(m01, r1, m00 r0), z1 = fma(m11, r1, m10 r0))
template <class T, bool BLOCK>
__device__ __forceinline__ typename Vec2<T>::type precondition(const T *__restrict__ minv, int32_t i,
                                                               typename Vec2<T>::type rr)
{
    typedef typename Vec2<T>::type V;
    if (BLOCK) {
        const V m01 = reinterpret_cast<const V *>(minv)[2 * i], m23 = reinterpret_cast<const V *>(minv)[2 * i + 1];
        return mk2(fma(m01.y, rr.y, m01.x * rr.x), fma(m23.y, rr.y, m23.x * rr.x));
    }
    const V di = reinterpret_cast<const V *>(minv)[i];
    return mk2(rr.x * di.x, rr.y * di.y);
}

// x = 0, r = b*scale (converted to T), z = M r, p = z; b.b and r.z
template <class T, bool BLOCK>
__global__ void __launch_bounds__(kRedBlock) k_cg_init(int32_t n_nodes, const double *__restrict__ b, double scale,
                                                       const T *__restrict__ dinv, T *__restrict__ x,
                                                       T *__restrict__ r, T *__restrict__ z, T *__restrict__ p,
                                                       T *part, int64_t n_red, unsigned *ticket, CGScalarsT<T> *sc,
                                                       T rtol, int max_it)
{
    typedef typename Vec2<T>::type V;
    const int32_t i = blockIdx.x * kRedBlock + threadIdx.x;
    T v[2] = {T(0), T(0)};
    if (i < n_nodes) {
        const double2 b64 = reinterpret_cast<const double2 *>(b)[i];
        const V bb = mk2((T)(b64.x * scale), (T)(b64.y * scale));
        const V zz = precondition<T, BLOCK>(dinv, i, bb);
        reinterpret_cast<V *>(x)[i] = mk2(T(0), T(0));
        reinterpret_cast<V *>(r)[i] = bb;
        reinterpret_cast<V *>(z)[i] = zz;
        reinterpret_cast<V *>(p)[i] = zz;
        v[0] = fma(bb.y, bb.y, fma(bb.x, bb.x, T(0)));
        v[1] = fma(bb.y, zz.y, fma(bb.x, zz.x, T(0)));
    }
    if (block_partials<T, 2>(v, part, n_red, ticket)) {
        T o[2];
        final_reduce<T, 2>(part, n_red, o);
        if (threadIdx.x == 0) {
            sc->bb = o[0];
            sc->rz = o[1];
            sc->thr = (rtol * rtol) * o[0];
            sc->iters = 0;
            sc->status = 0;
            sc->max_it = max_it;
            sc->done = (o[0] == T(0)) ? 1 : (max_it <= 0 ? 1 : 0);
            if (o[0] != T(0) && max_it <= 0) sc->status = IPFEM_NONCONVERGED;
            *ticket = 0u;
        }
    }
}

// q = K p (free dofs), partial sums of p.q; last CTA: alpha = rz / pq.
// SORTED: thread t runs SELL row position t, i.e. node sell_node[t] of the
// same kRedBlock window, and its p.q term goes through shared memory back to
// the node's own slot, so the block tree adds in node order either way.
// PAT: block k of the row has column i + pat_off[pat_id[t] * kPatLen + k]
// (row stencils, L1-resident) instead of the column index stored with it;
// same blocks in the same order, so the result is the same bit for bit.
// FP32 layouts use slot pairs, FP64 layouts one slot per lane and block.
template <class T, bool SORTED, bool PAT>
__global__ void __launch_bounds__(kRedBlock) k_cg_spmv(int32_t n_nodes, const int64_t *__restrict__ slice_base,
                                                       const int32_t *__restrict__ rowlen,
                                                       const int32_t *__restrict__ sell_node,
                                                       const int32_t *__restrict__ scol,
                                                       const uint8_t *__restrict__ pat_id,
                                                       const int32_t *__restrict__ pat_off, const T *__restrict__ K,
                                                       const uint8_t *__restrict__ fixed, const T *__restrict__ p,
                                                       T *__restrict__ q, T *part, int64_t n_red, unsigned *ticket,
                                                       CGScalarsT<T> *sc)
{
    typedef typename Vec2<T>::type V;
    constexpr bool PAIR = sizeof(T) == 4;
    __shared__ T s_pq[1][kRedStage];
    const int32_t t = blockIdx.x * kRedBlock + threadIdx.x;
    // row metadata is loaded before the flag so that the two latencies overlap
    int32_t i = t, len = 0, pb = 0;
    int64_t base = 0;
    if (t < n_nodes) {
        if (SORTED) i = __ldg(&sell_node[t]);
        base = sell_row0<PAIR>(__ldg(&slice_base[t >> 5]), t & 31);
        len = __ldg(&rowlen[t]);
        if (PAT) pb = (int)__ldg(&pat_id[t]) * kPatLen;
    }
    pdl_wait();
    pdl_launch_dependents();
    if (*reinterpret_cast<volatile int *>(&sc->done)) return;
    T v = T(0);
    if (t < n_nodes) {
        const V *pv = reinterpret_cast<const V *>(p);
        const uint64_t keep = l2_policy_keep();
        T y0 = T(0), y1 = T(0);
#pragma unroll 4
        for (int k = 0; k < len; k++) {
            const int64_t s = base + sell_koff<PAIR>(k);
            const int32_t c = PAT ? i + __ldg(&pat_off[pb + k]) : __ldg(&scol[s]);
            T a00, a01, a10, a11;
            load_block(K, s, a00, a01, a10, a11);
            const V xx = ld_keep(&pv[c], keep);
            y0 = fma(a00, xx.x, y0);
            y0 = fma(a01, xx.y, y0);
            y1 = fma(a10, xx.x, y1);
            y1 = fma(a11, xx.y, y1);
        }
        if (fixed[2 * (size_t)i]) y0 = T(0);
        if (fixed[2 * (size_t)i + 1]) y1 = T(0);
        reinterpret_cast<V *>(q)[i] = mk2(y0, y1);
        const V pp = pv[i];
        v = fma(pp.y, y1, fma(pp.x, y0, T(0)));
    }
    // the node's own slot of the window (sorted rows are a permutation of it;
    // slots past the last node get the zeros of the threads past it)
    s_pq[0][red_stage(i - blockIdx.x * kRedBlock)] = v;
    __syncthreads();
    if (block_partials_staged<T, 1>(s_pq, part, n_red, ticket)) {
        T o[1];
        final_reduce<T, 1>(part, n_red, o);
        if (threadIdx.x == 0) {
            const T pq = o[0];
            sc->pq = pq;
            if (!(pq > T(0))) {
                sc->done = 1;
                sc->status = IPFEM_BREAKDOWN;
            } else {
                sc->alpha = sc->rz / pq;
            }
            *ticket = 0u;
        }
    }
}

// The same SpMV over the upper-only FP32 layout (row and transposed
// stencils): row i first adds its lower blocks (i, j < i), read as the
// transposes of their stored twins (j, i) in ascending j, then its stored
// blocks (i, c >= i) in ascending c, which is the full layout's column order,
// so q and p.q are the same bits.  The stored blocks are loaded through L2
// (not evict-first): the rows of the next two grid lines read them again as
// twins.
__global__ void __launch_bounds__(kRedBlock) k_cg_spmv_sym(int32_t n_nodes, const int64_t *__restrict__ slice_base,
                                                           const int32_t *__restrict__ rowlen,
                                                           const uint8_t *__restrict__ pat_id,
                                                           const int32_t *__restrict__ pat_off,
                                                           const uint8_t *__restrict__ tpat_id,
                                                           const int2 *__restrict__ tpat,
                                                           const int32_t *__restrict__ tpat_len,
                                                           const float *__restrict__ K, const uint8_t *__restrict__ fixed,
                                                           const float *__restrict__ p, float *__restrict__ q,
                                                           float *part, int64_t n_red, unsigned *ticket,
                                                           CGScalarsT<float> *sc)
{
    __shared__ float s_pq[1][kRedStage];
    const int32_t i = blockIdx.x * kRedBlock + threadIdx.x;
    int32_t len = 0, pb = 0, tl = 0, tb = 0;
    int64_t base = 0;
    if (i < n_nodes) {
        base = sell_row0<true>(__ldg(&slice_base[i >> 5]), i & 31);
        len = __ldg(&rowlen[i]);
        pb = (int)__ldg(&pat_id[i]) * kPatLen;
        const int t = __ldg(&tpat_id[i]);
        tl = __ldg(&tpat_len[t]);
        tb = t * kPatLen;
    }
    pdl_wait();
    pdl_launch_dependents();
    if (*reinterpret_cast<volatile int *>(&sc->done)) return;
    float v = 0.f;
    if (i < n_nodes) {
        const float2 *pv = reinterpret_cast<const float2 *>(p);
        const float4 *K4 = reinterpret_cast<const float4 *>(K);
        const uint64_t keep = l2_policy_keep();
        float y0 = 0.f, y1 = 0.f;
#pragma unroll 4
        for (int k = 0; k < tl; k++) {
            const int2 e = __ldg(&tpat[tb + k]);
            const int32_t j = i + e.x;
            const float4 a = transpose4(__ldcg(&K4[sym_twin_slot(slice_base, j, e.y)]));
            const float2 xx = ld_keep(&pv[j], keep);
            y0 = fmaf(a.x, xx.x, y0);
            y0 = fmaf(a.y, xx.y, y0);
            y1 = fmaf(a.z, xx.x, y1);
            y1 = fmaf(a.w, xx.y, y1);
        }
#pragma unroll 4
        for (int k = 0; k < len; k++) {
            const int32_t c = i + __ldg(&pat_off[pb + k]);
            const float4 a = __ldcg(&K4[base + sell_koff<true>(k)]);
            const float2 xx = ld_keep(&pv[c], keep);
            y0 = fmaf(a.x, xx.x, y0);
            y0 = fmaf(a.y, xx.y, y0);
            y1 = fmaf(a.z, xx.x, y1);
            y1 = fmaf(a.w, xx.y, y1);
        }
        if (fixed[2 * (size_t)i]) y0 = 0.f;
        if (fixed[2 * (size_t)i + 1]) y1 = 0.f;
        reinterpret_cast<float2 *>(q)[i] = make_float2(y0, y1);
        const float2 pp = pv[i];
        v = fmaf(pp.y, y1, fmaf(pp.x, y0, 0.f));
    }
    s_pq[0][red_stage(threadIdx.x)] = v;
    __syncthreads();
    if (block_partials_staged<float, 1>(s_pq, part, n_red, ticket)) {
        float o[1];
        final_reduce<float, 1>(part, n_red, o);
        if (threadIdx.x == 0) {
            const float pq = o[0];
            sc->pq = pq;
            if (!(pq > 0.f)) {
                sc->done = 1;
                sc->status = IPFEM_BREAKDOWN;
            } else {
                sc->alpha = sc->rz / pq;
            }
            *ticket = 0u;
        }
    }
}

// x += alpha p, r -= alpha q, z = M r; partials of r.r and r.z;
// last CTA: convergence test, beta
template <class T, bool BLOCK>
__global__ void __launch_bounds__(kRedBlock) k_cg_update(int32_t n_nodes, const T *__restrict__ p,
                                                         const T *__restrict__ q, const T *__restrict__ dinv,
                                                         T *__restrict__ x, T *__restrict__ r, T *__restrict__ z,
                                                         T *part, int64_t n_red, unsigned *ticket, CGScalarsT<T> *sc)
{
    typedef typename Vec2<T>::type V;
    const int32_t i = blockIdx.x * kRedBlock + threadIdx.x;
    // p, x and r (not written by the SpMV) before the wait, q after it
    V pp, qq, xx, rr;
    if (i < n_nodes) {
        pp = reinterpret_cast<const V *>(p)[i];
        xx = reinterpret_cast<V *>(x)[i];
        rr = reinterpret_cast<V *>(r)[i];
    }
    pdl_wait();
    pdl_launch_dependents();
    if (i < n_nodes) qq = reinterpret_cast<const V *>(q)[i];
    if (*reinterpret_cast<volatile int *>(&sc->done)) return;
    const T alpha = *reinterpret_cast<volatile T *>(&sc->alpha);
    T v[2] = {T(0), T(0)};
    if (i < n_nodes) {
        xx.x = fma(alpha, pp.x, xx.x);
        xx.y = fma(alpha, pp.y, xx.y);
        rr.x = fma(-alpha, qq.x, rr.x);
        rr.y = fma(-alpha, qq.y, rr.y);
        const V zz = precondition<T, BLOCK>(dinv, i, rr);
        reinterpret_cast<V *>(x)[i] = xx;
        reinterpret_cast<V *>(r)[i] = rr;
        reinterpret_cast<V *>(z)[i] = zz;
        v[0] = fma(rr.y, rr.y, fma(rr.x, rr.x, T(0)));
        v[1] = fma(rr.y, zz.y, fma(rr.x, zz.x, T(0)));
    }
    if (block_partials<T, 2>(v, part, n_red, ticket)) {
        T o[2];
        final_reduce<T, 2>(part, n_red, o);
        if (threadIdx.x == 0) {
            const T rr = o[0], rzn = o[1];
            sc->rr = rr;
            sc->iters += 1;
            if (rr <= sc->thr) {
                sc->done = 1;
            } else if (sc->iters >= sc->max_it) {
                sc->done = 1;
                sc->status = IPFEM_NONCONVERGED;
            } else {
                sc->beta = rzn / sc->rz;
                sc->rz = rzn;
            }
            *ticket = 0u;
        }
    }
}

// p = z + beta p, kPupNodes nodes per thread (strided by the CTA size) so that
// each thread has several loads in flight: the kernel moves 48 bytes per node
// and is bound by memory latency, not bandwidth, at one node per thread
constexpr int kPupNodes = 4;

template <class T>
__global__ void __launch_bounds__(kRedBlock) k_cg_pupdate(int32_t n_nodes, const T *__restrict__ z,
                                                          T *__restrict__ p, const CGScalarsT<T> *sc)
{
    typedef typename Vec2<T>::type V;
    const int32_t i0 = blockIdx.x * (kRedBlock * kPupNodes) + threadIdx.x;
    // p (not written by the update) before the wait, z after it
    V pp[kPupNodes], zz[kPupNodes];
#pragma unroll
    for (int j = 0; j < kPupNodes; j++)
        if (i0 + j * kRedBlock < n_nodes) pp[j] = reinterpret_cast<V *>(p)[i0 + j * kRedBlock];
    pdl_wait();
    pdl_launch_dependents();
#pragma unroll
    for (int j = 0; j < kPupNodes; j++)
        if (i0 + j * kRedBlock < n_nodes) zz[j] = reinterpret_cast<const V *>(z)[i0 + j * kRedBlock];
    if (*reinterpret_cast<const volatile int *>(&sc->done)) return;
    const T beta = *reinterpret_cast<const volatile T *>(&sc->beta);
#pragma unroll
    for (int j = 0; j < kPupNodes; j++)
        if (i0 + j * kRedBlock < n_nodes) {
            pp[j].x = fma(beta, pp[j].x, zz[j].x);
            pp[j].y = fma(beta, pp[j].y, zz[j].y);
            reinterpret_cast<V *>(p)[i0 + j * kRedBlock] = pp[j];
        }
}

__global__ void __launch_bounds__(kRedBlock) k_dot(int32_t n_nodes, const double *__restrict__ a,
                                                   const double *__restrict__ b, double *part, int64_t n_red,
                                                   unsigned *ticket, double *out)
{
    const int32_t i = blockIdx.x * kRedBlock + threadIdx.x;
    double v[1] = {0.0};
    if (i < n_nodes) {
        const double2 aa = reinterpret_cast<const double2 *>(a)[i];
        const double2 bb = reinterpret_cast<const double2 *>(b)[i];
        v[0] = fma(aa.y, bb.y, fma(aa.x, bb.x, 0.0));
    }
    if (block_partials<double, 1>(v, part, n_red, ticket)) {
        double o[1];
        final_reduce<double, 1>(part, n_red, o);
        if (threadIdx.x == 0) {
            *out = o[0];
            *ticket = 0u;
        }
    }
}

__global__ void k_add(int64_t n, double *__restrict__ u, const double *__restrict__ du)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) u[i] = u[i] + du[i];
}

// secant predictor of a load step: u <- u + ratio (u - u_prev), u_prev <- the old u
__global__ void k_predict(int64_t n, double *__restrict__ u, double *__restrict__ u_prev, double ratio)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) {
        const double ui = u[i];
        u[i] = fma(ratio, ui - u_prev[i], ui);
        u_prev[i] = ui;
    }
}

// FP64 FMA issue-rate probe: 8 independent fma chains per thread, bounded loop
__global__ void __launch_bounds__(256) k_fp64_probe(double *out, int iters, double a, double b)
{
    double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
#pragma unroll 1
    for (int i = 0; i < iters; i++) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
}

void launch_fp64_probe(ipfem_ctx *c, double *d_out, int grid, int iters)
{
    k_fp64_probe<<<grid, 256, 0, c->stream>>>(d_out, iters, 0.999, 0.001);
}

// t = alpha * x, u = u + t (two rounded operations, in this order)
__global__ void k_scale_add(int64_t n, double *__restrict__ u, const double *__restrict__ x, double alpha,
                            double *__restrict__ t)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double ti = alpha * x[i];
    t[i] = ti;
    u[i] = u[i] + ti;
}

__global__ void k_add_scaled32(int64_t n, double *__restrict__ u, const float *__restrict__ x, double scale)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) u[i] = fma(scale, (double)x[i], u[i]);
}

static unsigned grid_nodes(const ipfem_ctx *c)
{
    return (unsigned)((c->s.n_nodes + kRedBlock - 1) / kRedBlock);
}

void launch_cg_init(ipfem_ctx *c, const double *d_b, double rtol, int max_it)
{
    const bool blk = c->preconditioner == IPFEM_PREC_BLOCK_JACOBI;
    (blk ? k_cg_init<double, true> : k_cg_init<double, false>)<<<grid_nodes(c), kRedBlock, 0, c->stream>>>(
        c->s.n_nodes, d_b, 1.0, blk ? c->d_binv : c->d_dinv, c->d_x, c->d_r,
                                                                  c->d_z, c->d_p, c->d_part, c->n_red,
                                                                  c->d_counters + 0, c->d_sc, rtol, max_it);
}

static unsigned grid_pupdate(const ipfem_ctx *c)
{
    return (unsigned)((c->s.n_nodes + kRedBlock * kPupNodes - 1) / (kRedBlock * kPupNodes));
}

template <class T>
void launch_spmv(ipfem_ctx *c, const SellDev &L, const T *K, const T *p, T *q, T *part, unsigned *ticket,
                 CGScalarsT<T> *sc)
{
    if constexpr (sizeof(T) == 4) {
        if (L.sym) {
            launch_pdl(k_cg_spmv_sym, grid_nodes(c), kRedBlock, c->stream, c->s.n_nodes,
                       (const int64_t *)L.slice_base, (const int32_t *)L.rowlen, (const uint8_t *)L.pat_id,
                       (const int32_t *)L.pat_off, (const uint8_t *)L.tpat_id, (const int2 *)L.tpat,
                       (const int32_t *)L.tpat_len, (const float *)K, (const uint8_t *)c->d_fixed, (const float *)p,
                       (float *)q, (float *)part, c->n_red, ticket, (CGScalarsT<float> *)sc);
            return;
        }
    }
    const bool pat = use_row_stencils(c, L);
    auto kern = L.sorted ? (pat ? k_cg_spmv<T, true, true> : k_cg_spmv<T, true, false>)
                         : (pat ? k_cg_spmv<T, false, true> : k_cg_spmv<T, false, false>);
    launch_pdl(kern, grid_nodes(c), kRedBlock, c->stream, c->s.n_nodes, (const int64_t *)L.slice_base,
               (const int32_t *)L.rowlen, (const int32_t *)L.sell_node, (const int32_t *)L.sell_col,
               (const uint8_t *)L.pat_id, (const int32_t *)L.pat_off, (const T *)K, (const uint8_t *)c->d_fixed,
               (const T *)p, q, part, c->n_red, ticket, sc);
}

void launch_cg_iteration(ipfem_ctx *c)
{
    const unsigned g = grid_nodes(c);
    launch_spmv<double>(c, c->dsell, c->d_K, c->d_p, c->d_q, c->d_part, c->d_counters + 1, c->d_sc);
    const bool blk = c->preconditioner == IPFEM_PREC_BLOCK_JACOBI;
    launch_pdl(blk ? k_cg_update<double, true> : k_cg_update<double, false>, g, kRedBlock, c->stream, c->s.n_nodes,
               (const double *)c->d_p, (const double *)c->d_q, (const double *)(blk ? c->d_binv : c->d_dinv), c->d_x,
               c->d_r, c->d_z, c->d_part, c->n_red, c->d_counters + 2, c->d_sc);
    launch_pdl(k_cg_pupdate<double>, grid_pupdate(c), kRedBlock, c->stream, c->s.n_nodes,
               (const double *)c->d_z, c->d_p, (const CGScalarsT<double> *)c->d_sc);
}

void launch_cg_spmv_only(ipfem_ctx *c)
{
    launch_spmv<double>(c, c->dsell, c->d_K, c->d_p, c->d_q, c->d_part, c->d_counters + 1, c->d_sc);
}

void launch_cg32_init(ipfem_ctx *c, const double *d_b, double scale, float rtol, int max_it)
{
    MixedBuffers &m = c->mx;
    const bool blk = c->preconditioner == IPFEM_PREC_BLOCK_JACOBI;
    (blk ? k_cg_init<float, true> : k_cg_init<float, false>)<<<grid_nodes(c), kRedBlock, 0, c->stream>>>(
        c->s.n_nodes, d_b, scale, blk ? m.binv : m.dinv, m.x, m.r, m.z,
                                                                 m.p, m.part, c->n_red, c->d_counters + 4, m.sc,
                                                                 rtol, max_it);
}

void launch_cg32_iteration(ipfem_ctx *c)
{
    MixedBuffers &m = c->mx;
    const unsigned g = grid_nodes(c);
    launch_spmv<float>(c, fp32_layout(c), fp32_values(c), m.p, m.q, m.part, c->d_counters + 5, m.sc);
    const bool blk = c->preconditioner == IPFEM_PREC_BLOCK_JACOBI;
    launch_pdl(blk ? k_cg_update<float, true> : k_cg_update<float, false>, g, kRedBlock, c->stream, c->s.n_nodes,
               (const float *)m.p, (const float *)m.q, (const float *)(blk ? m.binv : m.dinv), m.x, m.r, m.z, m.part,
               c->n_red, c->d_counters + 6, m.sc);
    launch_pdl(k_cg_pupdate<float>, grid_pupdate(c), kRedBlock, c->stream, c->s.n_nodes, (const float *)m.z,
               m.p, (const CGScalarsT<float> *)m.sc);
}

void launch_cg32_spmv_only(ipfem_ctx *c)
{
    MixedBuffers &m = c->mx;
    launch_spmv<float>(c, fp32_layout(c), fp32_values(c), m.p, m.q, m.part, c->d_counters + 5, m.sc);
}

void launch_cg32_pupdate_only(ipfem_ctx *c)
{
    MixedBuffers &m = c->mx;
    k_cg_pupdate<float><<<grid_pupdate(c), kRedBlock, 0, c->stream>>>(c->s.n_nodes, m.z, m.p, m.sc);
}

void launch_add_scaled32(ipfem_ctx *c, double *d_u, const float *x, double scale)
{
    const int64_t n = c->s.neq;
    k_add_scaled32<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, d_u, x, scale);
}

void launch_dot(ipfem_ctx *c, const double *a, const double *b, double *d_out)
{
    k_dot<<<grid_nodes(c), kRedBlock, 0, c->stream>>>(c->s.n_nodes, a, b, c->d_part, c->n_red, c->d_counters + 3,
                                                      d_out);
}

void launch_scale_add(ipfem_ctx *c, double *d_u, const double *d_x, double alpha, double *d_t)
{
    const int64_t n = c->s.neq;
    k_scale_add<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, d_u, d_x, alpha, d_t);
}

void launch_axpy_u(ipfem_ctx *c, double *d_u, const double *d_du)
{
    const int64_t n = c->s.neq;
    k_add<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, d_u, d_du);
}

void launch_predict(ipfem_ctx *c, double *d_u, double *d_u_prev, double ratio)
{
    const int64_t n = c->s.neq;
    k_predict<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, d_u, d_u_prev, ratio);
}

// ---------------------------------------------------------------------------
// Canonical dot product without device allocation.
//
// Some callers of this library cannot allocate device memory: a host
// application that hands every device byte out of its own preallocated pool
// (so that a solve never triggers cudaMalloc, which synchronises the device
// and fragments the pool), or a latency-critical pipeline that must never
// stall on an allocation.  For them the dot kernel above
// runs with its scratch (the per-CTA partial sums and the last-CTA ticket) in
// the file-scope array below instead of in a context's buffers.  The array
// holds kNoAllocMaxPartials partials (512 KiB), so vectors of up to
// 2 * 256 * kNoAllocMaxPartials doubles are accepted; every GPU that loads the
// library keeps the array until the process exits.
// ---------------------------------------------------------------------------
constexpr int64_t kNoAllocMaxPartials = 65536;

struct NoAllocScratch {
    double partials[kNoAllocMaxPartials];
    unsigned ticket;
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

}  // namespace ipfem

extern "C" ipfem_status ipfem_dot_noalloc(const double *d_a, const double *d_b, int64_t n, double *d_out,
                                          void *stream)
{
    using namespace ipfem;
    // every argument is checked before the first CUDA call: a rejected call
    // touches neither the device nor the stream
    if (!d_a || !d_b || !d_out || n < 0 || (n & 1)) {
        set_thread_error("ipfem_dot_noalloc: null pointer, negative or odd length");
        return IPFEM_INVALID;
    }
    // the kernel reads the vectors as pairs of doubles (16-byte loads)
    if ((reinterpret_cast<uintptr_t>(d_a) | reinterpret_cast<uintptr_t>(d_b)) & 15u) {
        set_thread_error("ipfem_dot_noalloc: d_a and d_b must be 16-byte aligned");
        return IPFEM_INVALID;
    }
    if (reinterpret_cast<uintptr_t>(d_out) & 7u) {
        set_thread_error("ipfem_dot_noalloc: d_out must be 8-byte aligned");
        return IPFEM_INVALID;
    }
    const int64_t n_nodes = n / 2;
    const int64_t n_red = (n_nodes + kRedBlock - 1) / kRedBlock;
    if (n_red > kNoAllocMaxPartials) {
        set_thread_error("ipfem_dot_noalloc: length " + std::to_string(n) + " exceeds the maximum of " +
                         std::to_string(2 * kRedBlock * kNoAllocMaxPartials) + " doubles");
        return IPFEM_INVALID;
    }
    // The host-side name of the array is not a device address: ask the
    // runtime for the address in the current device's context.  The lookup
    // allocates nothing; it is repeated on every call so that a context
    // created anew (after cudaDeviceReset, or on another device) is never
    // given a stale address.
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        set_thread_error(std::string("ipfem_dot_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
        return e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ? IPFEM_NO_DEVICE : IPFEM_CUDA;
    }
    NoAllocScratch *scr = static_cast<NoAllocScratch *>(p);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (n_nodes == 0) {
        e = cudaMemsetAsync(d_out, 0, sizeof(double), st);
    } else {
        // the array keeps the previous call's contents: the ticket must start at 0
        e = cudaMemsetAsync(&scr->ticket, 0, sizeof(unsigned), st);
        if (e == cudaSuccess) {
            k_dot<<<(unsigned)n_red, kRedBlock, 0, st>>>((int32_t)n_nodes, d_a, d_b, scr->partials, n_red,
                                                         &scr->ticket, d_out);
            e = cudaGetLastError();
        }
    }
    if (e != cudaSuccess) {
        set_thread_error(std::string("ipfem_dot_noalloc: ") + cudaGetErrorString(e));
        return IPFEM_CUDA;
    }
    return IPFEM_OK;
}
