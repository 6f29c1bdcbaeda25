// Element-block kernels of the residual and tangent assembly.
//
//  k_gather_strain   TPZNumericalIntegrator::Multiply (TPZNumericalIntegrator.cpp:25-37):
//                    gather of element dofs + B*u, fused.  The element blocks of
//                    a tile are staged in shared memory by one bulk (TMA) copy.
//  k_stress_residual TPZNumericalIntegrator::MultiplyTranspose (…cpp:54-78), first
//                    half: f_e = -B^T (w sigma) per element, blocks TMA-staged.
//  k_color_reduce    second half: the colour-slab scatter and pairwise slab
//                    reduction of the reference, evaluated per node as a
//                    gather over the (at most one per colour) incident elements,
//                    in the reference's pairing order; + the load vector
//                    f0 + lambda*df (k_load_vector, once per load factor) and
//                    Dirichlet masking (TPZElastoPlasticIntPointsStructMatrix.cpp:137-154).
//  k_gather_strain32, k_stress_residual32
//                    the same two element kernels in FP32 for the mixed
//                    precision's FP32 residuals, on tiles of 32 elements.
//  k_stiffness       TPZNumericalIntegrator::KAssembly (…cpp:131-214) and
//                    MatrixAssembleKernel (KernelsMatrixAssemble.h:24-57): one warp
//                    per element, K_e = sum_q B_q^T (w Dep_q) B_q (upper triangle),
//                    added colour by colour into the nodal 2x2 block matrix.
//
// Element blocks are stored compactly: dphi[e][q][d][n] = d(phi_n)/d(x_d) at
// point q (the reference's fStorage holds the same numbers in a (3 nq x 2 nn)
// block with structural zeros).  Products use fma in the order of the
// reference's row-major block traversal; skipped terms are exact zeros.
// Every kernel is instantiated for the element orders P = 1, 2, 3 (the
// reference builds one order per binary, KernelsMatrixAssemble.h:3-12):
// nn = nq = (P+1)^2 connects and Gauss points, nd = 2 nn dofs per element.
#include <algorithm>

#include "ipfem_internal.h"
#include "tma.cuh"

namespace ipfem {

template <int P>
struct Elem {
    static constexpr int N1 = P + 1, NN = N1 * N1, NQ = N1 * N1, ND = 2 * NN;
    static constexpr int NB = NQ * 2 * NN;                    // compact block values per element
    static constexpr int kGatherTile = P == 1 ? 64 : (P == 2 ? 32 : 8);   // elements per CTA
    static constexpr int kResTile = P == 1 ? 32 : (P == 2 ? 16 : 8);      // elements per CTA
};
static_assert(Elem<1>::NB * 8 % 16 == 0 && Elem<2>::NB * 8 % 16 == 0 && Elem<3>::NB * 8 % 16 == 0,
              "bulk copies of whole FP64 element blocks need 16-byte multiples");

// The plain path's strain gather (bit-exact with the oracle).
template <class T, int P>
__global__ void __launch_bounds__(Elem<P>::kGatherTile * Elem<P>::NQ)
k_gather_strain(int32_t n_el, int64_t n_ip, const T *__restrict__ dphi, const int32_t *__restrict__ dofs,
                const double *__restrict__ u, T *__restrict__ strain, int *__restrict__ err)
{
    typedef Elem<P> E;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    T *s_dn = reinterpret_cast<T *>(smem + 128);
    T *s_u = s_dn + E::kGatherTile * E::NB;
    const int32_t e0 = blockIdx.x * E::kGatherTile;
    const int ne = min(E::kGatherTile, n_el - e0);
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t bytes = (uint32_t)ne * E::NB * (uint32_t)sizeof(T);
        mbar_expect_tx(bar, bytes);
        bulk_g2s(s_dn, dphi + (size_t)e0 * E::NB, bytes, bar);
    }
    for (int k = threadIdx.x; k < ne * E::ND; k += blockDim.x)
        s_u[k] = __ldg(&u[__ldg(&dofs[(size_t)e0 * E::ND + k])]);
    const bool ok = mbar_wait_bounded(bar, 0);
    __syncthreads();
    if (!ok) {
        if (threadIdx.x == 0) atomicExch(err, kErrBulkWait);
        return;
    }
    const int el = threadIdx.x / E::NQ, q = threadIdx.x % E::NQ;
    if (el >= ne) return;
    const T *dx = s_dn + el * E::NB + q * 2 * E::NN;
    const T *dy = dx + E::NN;
    const T *ue = s_u + el * E::ND;
    T exx = T(0), gxy = T(0), eyy = T(0);
#pragma unroll
    for (int n = 0; n < E::NN; n++) exx = fma(dx[n], ue[2 * n], exx);
#pragma unroll
    for (int n = 0; n < E::NN; n++) {
        gxy = fma(dy[n], ue[2 * n], gxy);
        gxy = fma(dx[n], ue[2 * n + 1], gxy);
    }
#pragma unroll
    for (int n = 0; n < E::NN; n++) eyy = fma(dy[n], ue[2 * n + 1], eyy);
    const int64_t ip = (int64_t)(e0 + el) * E::NQ + q;
    strain[ip] = exx;
    strain[n_ip + ip] = gxy;
    strain[2 * n_ip + ip] = eyy;
}

// The plain path's element forces (bit-exact with the oracle).
template <class V, int P>
__global__ void __launch_bounds__(Elem<P>::kResTile * Elem<P>::ND)
k_stress_residual(int32_t n_el, int64_t n_ip, const V *__restrict__ dphi, const V *__restrict__ sigma_w,
                  V *__restrict__ fe, int *__restrict__ err)
{
    typedef Elem<P> E;
    constexpr int T = E::kResTile;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    V *s_dn = reinterpret_cast<V *>(smem + 128);
    V *s_sig = s_dn + T * E::NB;                       // [3][T*nq]
    const int32_t e0 = blockIdx.x * T;
    const int ne = min(T, n_el - e0);
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t bytes = (uint32_t)ne * E::NB * (uint32_t)sizeof(V);
        mbar_expect_tx(bar, bytes);
        bulk_g2s(s_dn, dphi + (size_t)e0 * E::NB, bytes, bar);
    }
    const int npt = ne * E::NQ;
    const int64_t ip0 = (int64_t)e0 * E::NQ;
    for (int k = threadIdx.x; k < 3 * npt; k += blockDim.x) {
        const int cmp = k / npt, i = k - cmp * npt;
        s_sig[cmp * T * E::NQ + i] = sigma_w[cmp * n_ip + ip0 + i];
    }
    const bool ok = mbar_wait_bounded(bar, 0);
    __syncthreads();
    if (!ok) {
        if (threadIdx.x == 0) atomicExch(err, kErrBulkWait);
        return;
    }
    const int el = threadIdx.x / E::ND, j = threadIdx.x % E::ND;
    if (el >= ne) return;
    const int n = j >> 1;
    const V *dn = s_dn + el * E::NB;
    // x-dof: dNx*sxx + dNy*sxy per point; y-dof: dNx*sxy + dNy*syy.  The two
    // stress rows are selected by pointer so the warp does not diverge.
    const V *s1 = s_sig + (j & 1) * T * E::NQ + el * E::NQ;
    const V *s2 = s1 + T * E::NQ;
    V acc = V(0);
#pragma unroll
    for (int q = 0; q < E::NQ; q++) {
        acc = fma(dn[q * 2 * E::NN + n], s1[q], acc);
        acc = fma(dn[q * 2 * E::NN + E::NN + n], s2[q], acc);
    }
    fe[(size_t)(e0 + el) * E::ND + j] = -acc;
}

// ---- FP32 residual kernels (IPFEM_MIXED with FP32 residuals) ----------------
// One CTA per tile of kTile32 = 32 elements.  The tile's blocks arrive in one
// bulk copy, laid out [d][n][element][q] with the point index padded to an odd
// stride QS: the gather's threads (one per point, q fastest) and the stress
// kernel's threads (one per node, element fastest) both read 32 different
// banks per warp.  Every output keeps the fma order of the element-major
// kernels above.

// odd stride (in words) of the per-element point rows
template <int N> struct OddStride { static constexpr int value = N | 1; };
// float2 rows: 8-byte words at a stride that keeps the 16 lanes of each
// half-warp phase on distinct bank pairs
template <int N> struct PairStride { static constexpr int value = (N % 4 == 0) ? N + 2 : N; };
// words of one tile of FP32 residual blocks
template <int P> struct Tile32 {
    static constexpr int QS = OddStride<Elem<P>::NQ>::value;
    static constexpr int words = 2 * Elem<P>::NN * kTile32 * QS;
    static_assert(words * 4 % 16 == 0, "tiles start on 16-byte boundaries and are bulk-copied whole");
};

template <int P>
__global__ void k_tile_blocks32(int32_t n_el, int64_t total, const double *__restrict__ dphi,
                                float *__restrict__ dphiT)
{
    typedef Elem<P> E;
    constexpr int QS = Tile32<P>::QS, W = Tile32<P>::words;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total; k += (int64_t)gridDim.x * blockDim.x) {
        const int o = (int)(k % W);
        const int q = o % QS, el = (o / QS) % kTile32, dn = o / (QS * kTile32);
        const int d = dn / E::NN, n = dn - d * E::NN;
        const int64_t e = (k / W) * kTile32 + el;
        dphiT[k] = (q < E::NQ && e < n_el) ? (float)dphi[((e * E::NQ + q) * 2 + d) * E::NN + n] : 0.0f;
    }
}

// strain of every point of the tile: one thread per point (q fastest), so the
// strains leave in coalesced rows.  Each displacement is taken relative to the
// element's first connect (same component), formed in FP64 before rounding.
// The strain of a rigid translation is zero, so the strain is unchanged, but
// the rounded values carry the variation across the element instead of the
// far-field displacement, which is orders of magnitude larger.
template <int P>
__global__ void __launch_bounds__(kTile32 * Elem<P>::NQ)
k_gather_strain32(int32_t n_el, int64_t n_ip, const float *__restrict__ dphiT, const int32_t *__restrict__ dofs,
                  const double *__restrict__ u, float *__restrict__ strain, int *__restrict__ err)
{
    typedef Elem<P> E;
    constexpr int T = kTile32, QS = Tile32<P>::QS, W = Tile32<P>::words;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    float *s_dn = reinterpret_cast<float *>(smem + 128);   // [2][NN][T][QS]
    float *s_u = s_dn + W;                                  // [T][ND]
    const int32_t e0 = blockIdx.x * T;
    const int ne = min(T, n_el - e0);
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_expect_tx(bar, W * sizeof(float));
        bulk_g2s(s_dn, dphiT + (size_t)blockIdx.x * W, W * sizeof(float), bar);
    }
    // the tile's 2 NN T displacements, two per thread (ND = 2 NQ), with both
    // threads' index loads issued before their displacement loads
    static_assert(E::ND == 2 * E::NQ, "two staged displacements per thread");
    const int32_t *de = dofs + (size_t)e0 * E::ND;
    const int lim = ne * E::ND;
    const int k0 = threadIdx.x, k1 = threadIdx.x + T * E::NQ;
    int32_t i0 = 0, j0 = 0, i1 = 0, j1 = 0;
    if (k0 < lim) {
        i0 = __ldg(&de[k0]);
        j0 = __ldg(&de[k0 - k0 % E::ND + (k0 & 1)]);
    }
    if (k1 < lim) {
        i1 = __ldg(&de[k1]);
        j1 = __ldg(&de[k1 - k1 % E::ND + (k1 & 1)]);
    }
    double a0 = 0.0, b0 = 0.0, a1 = 0.0, b1 = 0.0;
    if (k0 < lim) {
        a0 = __ldg(&u[i0]);
        b0 = __ldg(&u[j0]);
    }
    if (k1 < lim) {
        a1 = __ldg(&u[i1]);
        b1 = __ldg(&u[j1]);
    }
    if (k0 < lim) s_u[k0] = (float)(a0 - b0);
    if (k1 < lim) s_u[k1] = (float)(a1 - b1);
    const bool ok = mbar_wait_bounded(bar, 0);
    __syncthreads();
    if (!ok) {
        if (threadIdx.x == 0) atomicExch(err, kErrBulkWait);
        return;
    }
    const int el = threadIdx.x / E::NQ, q = threadIdx.x - el * E::NQ;
    if (el >= ne) return;
    const float *dx = s_dn + el * QS + q;                   // dx[n T QS]
    const float *dy = dx + E::NN * T * QS;
    const float *ue = s_u + el * E::ND;
    float exx = 0.0f, gxy = 0.0f, eyy = 0.0f;
#pragma unroll
    for (int n = 0; n < E::NN; n++) exx = fmaf(dx[n * T * QS], ue[2 * n], exx);
#pragma unroll
    for (int n = 0; n < E::NN; n++) {
        gxy = fmaf(dy[n * T * QS], ue[2 * n], gxy);
        gxy = fmaf(dx[n * T * QS], ue[2 * n + 1], gxy);
    }
#pragma unroll
    for (int n = 0; n < E::NN; n++) eyy = fmaf(dy[n * T * QS], ue[2 * n + 1], eyy);
    const int64_t ip = (int64_t)e0 * E::NQ + threadIdx.x;
    strain[ip] = exx;
    strain[n_ip + ip] = gxy;
    strain[2 * n_ip + ip] = eyy;
}

// element forces -B^T (w sigma) of the tile: thread (node, element), element
// fastest, both components, each summed over the points in the element-major
// kernel's order
template <int P>
__global__ void __launch_bounds__(kTile32 * Elem<P>::NN)
k_stress_residual32(int32_t n_el, int64_t n_ip, const float *__restrict__ dphiT, const float *__restrict__ sigma_w,
                    float *__restrict__ fe, int *__restrict__ err)
{
    typedef Elem<P> E;
    constexpr int T = kTile32, QS = Tile32<P>::QS, W = Tile32<P>::words, FS = PairStride<E::ND>::value;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
    float *s_dn = reinterpret_cast<float *>(smem + 128);   // [2][NN][T][QS]
    float *s_sig = s_dn + W;                                // [3][T][QS]
    float *s_fe = s_sig + 3 * T * QS;                       // [T][FS]
    const int32_t e0 = blockIdx.x * T;
    const int ne = min(T, n_el - e0);
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_expect_tx(bar, W * sizeof(float));
        bulk_g2s(s_dn, dphiT + (size_t)blockIdx.x * W, W * sizeof(float), bar);
    }
    // the tile's weighted stresses: one point per thread (NN = NQ), its three
    // components loaded together
    static_assert(E::NN == E::NQ, "one staged point per thread");
    {
        const int t = threadIdx.x;
        if (t < ne * E::NQ) {
            const int64_t ip = (int64_t)e0 * E::NQ + t;
            const float a = sigma_w[ip], b = sigma_w[n_ip + ip], c = sigma_w[2 * n_ip + ip];
            const int e = t / E::NQ, q = t - e * E::NQ;
            s_sig[e * QS + q] = a;
            s_sig[(T + e) * QS + q] = b;
            s_sig[(2 * T + e) * QS + q] = c;
        }
    }
    const bool ok = mbar_wait_bounded(bar, 0);
    __syncthreads();
    if (!ok) {
        if (threadIdx.x == 0) atomicExch(err, kErrBulkWait);
        return;
    }
    const int el = threadIdx.x % T, n = threadIdx.x / T;
    const float *dnx = s_dn + (n * T + el) * QS;            // dNx at q: dnx[q], dNy: dnx[NN T QS + q]
    const float *dny = dnx + E::NN * T * QS;
    const float *sxx = s_sig + el * QS, *sxy = sxx + T * QS, *syy = sxy + T * QS;
    float fx = 0.0f, fy = 0.0f;
#pragma unroll
    for (int q = 0; q < E::NQ; q++) {
        const float nx = dnx[q], ny = dny[q], txy = sxy[q];
        fx = fmaf(nx, sxx[q], fx);
        fx = fmaf(ny, txy, fx);
        fy = fmaf(nx, txy, fy);
        fy = fmaf(ny, syy[q], fy);
    }
    *reinterpret_cast<float2 *>(&s_fe[el * FS + 2 * n]) = make_float2(-fx, -fy);
    __syncthreads();
    float2 *out = reinterpret_cast<float2 *>(fe + (size_t)e0 * E::ND);
    for (int k = threadIdx.x; k < ne * E::NN; k += blockDim.x) {
        const int e = k / E::NN, nn = k - e * E::NN;
        out[k] = *reinterpret_cast<const float2 *>(&s_fe[e * FS + 2 * nn]);
    }
}

// Per node: contributions of the incident element of each colour (0 if none),
// summed in the reference's pairwise slab order
// (TPZNumericalIntegrator.cpp:69-77: slab k += slab (nc-ca)+k, nc -= ca).
template <class V> struct Pair;
template <> struct Pair<double> { typedef double2 type; };
template <> struct Pair<float> { typedef float2 type; };

// The reference's pairwise slab sum over NC colours, unrolled at compile time
// so that the per-colour sums stay in registers: step with ca = nc / 2 adds
// slab first + k (first = nc - ca) into slab k for k < ca, then nc -= ca.
template <int NC> struct SlabPairs {
    template <class V>
    __device__ static void run(V *sx, V *sy)
    {
        constexpr int ca = NC / 2, first = NC - ca;
#pragma unroll
        for (int k = 0; k < ca; k++) {
            sx[k] = sx[k] + sx[first + k];
            sy[k] = sy[k] + sy[first + k];
        }
        SlabPairs<NC - ca>::run(sx, sy);
    }
};
template <> struct SlabPairs<1> {
    template <class V> __device__ static void run(V *, V *) {}
};
template <> struct SlabPairs<0> {
    template <class V> __device__ static void run(V *, V *) {}
};

// V = float: the element forces of the FP32 residual, summed in FP32; the
// external load (FP64) is added to the FP32 sum in FP64.  NC = the number of
// colours.  The load vector and the Dirichlet flags are read before the
// incidence so that their latency overlaps the dependent element-force loads.
template <class V, int NC>
__global__ void __launch_bounds__(256) k_color_reduce(int32_t n_nodes, const int32_t *__restrict__ inc,
                                                      const V *__restrict__ fe, int with_load,
                                                      const double *__restrict__ lin,
                                                      const uint8_t *__restrict__ fixed,
                                                      double *__restrict__ res)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_nodes) return;
    double2 lv = make_double2(0.0, 0.0);
    uchar2 fx = make_uchar2(0, 0);
    if (with_load) {
        lv = __ldg(reinterpret_cast<const double2 *>(lin) + i);
        fx = __ldg(reinterpret_cast<const uchar2 *>(fixed) + i);
    }
    constexpr int NS = NC > 0 ? NC : 1;
    int32_t k[NS];
#pragma unroll
    for (int c = 0; c < NC; c++) k[c] = __ldg(&inc[(size_t)c * n_nodes + i]);
    V sx[NS], sy[NS];
    sx[0] = V(0);
    sy[0] = V(0);
#pragma unroll
    for (int c = 0; c < NC; c++) {
        sx[c] = V(0);
        sy[c] = V(0);
        if (k[c] >= 0) {
            const typename Pair<V>::type v = *reinterpret_cast<const typename Pair<V>::type *>(&fe[2 * (size_t)k[c]]);
            sx[c] = v.x;
            sy[c] = v.y;
        }
    }
    SlabPairs<NC>::run(sx, sy);
    double rx = (double)sx[0], ry = (double)sy[0];
    if (with_load) {
        rx = fx.x ? 0.0 : rx + lv.x;
        ry = fx.y ? 0.0 : ry + lv.y;
    }
    reinterpret_cast<double2 *>(res)[i] = make_double2(rx, ry);
}

// rhs_linear = f0 + lambda df (AssembleBoundaryData's fRhsLinear,
// TPZElastoPlasticIntPointsStructMatrix.cpp:156-167), once per load factor
__global__ void k_load_vector(int32_t neq, double lambda, const double *__restrict__ f0,
                              const double *__restrict__ df, double *__restrict__ lin)
{
    for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < neq; i += gridDim.x * blockDim.x)
        lin[i] = fma(lambda, df[i], f0[i]);
}

constexpr int kStiffWarps = 4;

// T = double: the plain tangent (bit-exact with the oracle); T = float: the
// FP32 tangent of the mixed-precision solve (blocks and w*Dep rounded to FP32,
// FP32 fma accumulation).
template <class T, int P>
__global__ void __launch_bounds__(kStiffWarps * 32) k_stiffness(int32_t n_in_color, const int32_t *__restrict__ els,
                                                                 int64_t n_ip, const T *__restrict__ dphi,
                                                                 const double *__restrict__ dep,
                                                                 const int32_t *__restrict__ el_blk,
                                                                 T *__restrict__ K)
{
    typedef Elem<P> E;
    constexpr int NE = E::ND * (E::ND + 1) / 2;   // upper-triangle entries
    constexpr int MM = (NE + 31) / 32;            // entries per lane
    __shared__ __align__(16) T s_dn[kStiffWarps][E::NB];
    __shared__ T s_D[kStiffWarps][E::NQ * 9];    // [q][9]
    __shared__ T s_DB[kStiffWarps][3 * E::ND];   // [3][nd]
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int32_t k = blockIdx.x * kStiffWarps + w;
    if (k >= n_in_color) return;              // warp-uniform
    const int32_t e = __ldg(&els[k]);
    const T *dn_g = dphi + (size_t)e * E::NB;
    for (int t = lane; t < E::NB; t += 32) s_dn[w][t] = __ldg(&dn_g[t]);
    for (int t = lane; t < 9 * E::NQ; t += 32) {
        const int cmp = t / E::NQ, q = t - cmp * E::NQ;
        s_D[w][q * 9 + cmp] = (T)__ldg(&dep[cmp * n_ip + (int64_t)e * E::NQ + q]);
    }
    __syncwarp();
    const T *dn = s_dn[w];
    // upper-triangle entries (a <= b, row-major order) owned by this lane
    int pa[MM], pb[MM];
#pragma unroll
    for (int m = 0; m < MM; m++) {
        int r = lane + 32 * m, a = 0;
        if (r < NE)
            while (r >= E::ND - a) {
                r -= E::ND - a;
                a++;
            }
        pa[m] = a;
        pb[m] = a + r;
    }
    T acc[MM];
#pragma unroll
    for (int m = 0; m < MM; m++) acc[m] = T(0);
#pragma unroll 1
    for (int q = 0; q < E::NQ; q++) {
        const T *D = &s_D[w][q * 9];
        const T *dx = dn + q * 2 * E::NN, *dy = dx + E::NN;
        for (int t = lane; t < 3 * E::ND; t += 32) {
            // x-dof column j: D[i][0] dNx + D[i][1] dNy; y-dof: D[i][1] dNx + D[i][2] dNy
            const int i = t / E::ND, j = t - i * E::ND, n = j >> 1, c0 = 3 * i + (j & 1);
            T sv = D[c0] * dx[n];
            sv = fma(D[c0 + 1], dy[n], sv);
            s_DB[w][t] = sv;
        }
        __syncwarp();
        const T *DB = s_DB[w];
#pragma unroll
        for (int m = 0; m < MM; m++) {
            const int p = lane + 32 * m;
            if (p < NE) {
                // x-dof row a: dNx DB[0][b] + dNy DB[1][b]; y-dof: dNx DB[1][b] + dNy DB[2][b]
                const int a = pa[m], b = pb[m], na = a >> 1, o = (a & 1) * E::ND + b;
                T t = acc[m];
                t = fma(dx[na], DB[o], t);
                t = fma(dy[na], DB[o + E::ND], t);
                acc[m] = t;
            }
        }
        __syncwarp();
    }
    const int32_t *eb = el_blk + (size_t)e * E::NN * E::NN;
#pragma unroll
    for (int m = 0; m < MM; m++) {
        const int p = lane + 32 * m;
        if (p < NE) {
            const int a = pa[m], b = pb[m];
            const int ma = a >> 1, ca = a & 1, nb = b >> 1, cb = b & 1;
            const T v = acc[m];
            if (ma == nb) {
                T *blk = K + 4 * (size_t)__ldg(&eb[ma * E::NN + ma]);
                blk[2 * ca + cb] = blk[2 * ca + cb] + v;
                if (ca != cb) blk[2 * cb + ca] = blk[2 * cb + ca] + v;
            } else {
                // an entry and its mirror; the upper-only FP32 layout stores
                // one of the two blocks (the other's map entry is -1)
                const int32_t s1 = __ldg(&eb[ma * E::NN + nb]), s2 = __ldg(&eb[nb * E::NN + ma]);
                if (s1 >= 0) {
                    T *b1 = K + 4 * (size_t)s1;
                    b1[2 * ca + cb] = b1[2 * ca + cb] + v;
                }
                if (s2 >= 0) {
                    T *b2 = K + 4 * (size_t)s2;
                    b2[2 * cb + ca] = b2[2 * cb + ca] + v;
                }
            }
        }
    }
}

// Jacobi inverses of the free diagonal entries and, when binv is given, the
// inverse of every nodal 2x2 diagonal block restricted to its free dofs
// (block Jacobi; det = a d - b c, entries d/det, -b/det, -c/det, a/det).
template <class T>
__global__ void k_jacobi(int32_t n_nodes, const int64_t *__restrict__ diag, const T *__restrict__ K,
                         const uint8_t *__restrict__ fixed, T *__restrict__ dinv, T *__restrict__ binv)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_nodes) return;
    const T *blk = K + 4 * (size_t)diag[i];
    const bool fx = fixed[2 * (size_t)i], fy = fixed[2 * (size_t)i + 1];
    dinv[2 * (size_t)i] = fx ? T(0) : T(1) / blk[0];
    dinv[2 * (size_t)i + 1] = fy ? T(0) : T(1) / blk[3];
    if (binv) {
        T m0 = T(0), m1 = T(0), m2 = T(0), m3 = T(0);
        if (!fx && !fy) {
            const T det = blk[0] * blk[3] - blk[1] * blk[2];
            m0 = blk[3] / det;
            m1 = -blk[1] / det;
            m2 = -blk[2] / det;
            m3 = blk[0] / det;
        } else if (!fx) {
            m0 = T(1) / blk[0];
        } else if (!fy) {
            m3 = T(1) / blk[3];
        }
        T *m = binv + 4 * (size_t)i;
        m[0] = m0;
        m[1] = m1;
        m[2] = m2;
        m[3] = m3;
    }
}

template <class T, int P>
static void gather_strain_p(ipfem_ctx *c, const T *dphi, const double *d_u, T *d_strain)
{
    typedef Elem<P> E;
    const Setup &s = c->s;
    const unsigned grid = (unsigned)((s.n_el + E::kGatherTile - 1) / E::kGatherTile);
    const size_t smem = 128 + (size_t)E::kGatherTile * (E::NB + E::ND) * sizeof(T);
    k_gather_strain<T, P><<<grid, E::kGatherTile * E::NQ, smem, c->stream>>>(s.n_el, s.n_ip, dphi, c->d_dofs, d_u,
                                                                              d_strain, c->d_err);
}

void launch_gather_strain(ipfem_ctx *c, const double *d_u, double *d_strain)
{
    switch (c->s.order) {
    case 1: gather_strain_p<double, 1>(c, c->d_dphi, d_u, d_strain); break;
    case 3: gather_strain_p<double, 3>(c, c->d_dphi, d_u, d_strain); break;
    default: gather_strain_p<double, 2>(c, c->d_dphi, d_u, d_strain); break;
    }
}

template <int P>
static void tile_blocks32_p(ipfem_ctx *c)
{
    const Setup &s = c->s;
    const int64_t total = (int64_t)((s.n_el + kTile32 - 1) / kTile32) * Tile32<P>::words;
    const unsigned grid = (unsigned)std::min<int64_t>((total + 255) / 256, 152 * 16);
    k_tile_blocks32<P><<<grid, 256, 0, c->stream>>>(s.n_el, total, c->d_dphi, c->mx.dphiT);
}

void launch_tile_blocks32(ipfem_ctx *c)
{
    switch (c->s.order) {
    case 1: tile_blocks32_p<1>(c); break;
    case 3: tile_blocks32_p<3>(c); break;
    default: tile_blocks32_p<2>(c); break;
    }
}

// dynamic shared memory above the default 48 KB (order 3 tiles) is opted into per kernel
template <class K>
static void allow_smem(K kern, size_t bytes)
{
    if (bytes > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <int P>
static void gather_strain32_p(ipfem_ctx *c, const double *d_u, float *d_strain)
{
    typedef Elem<P> E;
    const Setup &s = c->s;
    const unsigned grid = (unsigned)((s.n_el + kTile32 - 1) / kTile32);
    const size_t smem = 128 + (size_t)(Tile32<P>::words + kTile32 * E::ND) * sizeof(float);
    allow_smem(k_gather_strain32<P>, smem);
    k_gather_strain32<P><<<grid, kTile32 * E::NQ, smem, c->stream>>>(s.n_el, s.n_ip, c->mx.dphiT, c->d_dofs, d_u,
                                                                       d_strain, c->d_err);
}

void launch_gather_strain32(ipfem_ctx *c, const double *d_u, float *d_strain)
{
    switch (c->s.order) {
    case 1: gather_strain32_p<1>(c, d_u, d_strain); break;
    case 3: gather_strain32_p<3>(c, d_u, d_strain); break;
    default: gather_strain32_p<2>(c, d_u, d_strain); break;
    }
}

template <class V, int P>
static void stress_residual_p(ipfem_ctx *c, const V *dphi, const V *d_sigma_w, V *d_fe)
{
    typedef Elem<P> E;
    const Setup &s = c->s;
    const unsigned grid = (unsigned)((s.n_el + E::kResTile - 1) / E::kResTile);
    const size_t smem = 128 + (size_t)E::kResTile * (E::NB + 3 * E::NQ) * sizeof(V);
    k_stress_residual<V, P><<<grid, E::kResTile * E::ND, smem, c->stream>>>(s.n_el, s.n_ip, dphi, d_sigma_w, d_fe,
                                                                             c->d_err);
}

void launch_stress_residual(ipfem_ctx *c, const double *d_sigma_w, double *d_fe)
{
    switch (c->s.order) {
    case 1: stress_residual_p<double, 1>(c, c->d_dphi, d_sigma_w, d_fe); break;
    case 3: stress_residual_p<double, 3>(c, c->d_dphi, d_sigma_w, d_fe); break;
    default: stress_residual_p<double, 2>(c, c->d_dphi, d_sigma_w, d_fe); break;
    }
}

template <int P>
static void stress_residual32_p(ipfem_ctx *c, const float *d_sigma_w, float *d_fe)
{
    typedef Elem<P> E;
    const Setup &s = c->s;
    const unsigned grid = (unsigned)((s.n_el + kTile32 - 1) / kTile32);
    const size_t smem = 128 + (size_t)(Tile32<P>::words + 3 * kTile32 * Tile32<P>::QS +
                                       kTile32 * PairStride<E::ND>::value) * sizeof(float);
    allow_smem(k_stress_residual32<P>, smem);
    k_stress_residual32<P><<<grid, kTile32 * E::NN, smem, c->stream>>>(s.n_el, s.n_ip, c->mx.dphiT, d_sigma_w, d_fe,
                                                                         c->d_err);
}

void launch_stress_residual32(ipfem_ctx *c, const float *d_sigma_w, float *d_fe)
{
    switch (c->s.order) {
    case 1: stress_residual32_p<1>(c, d_sigma_w, d_fe); break;
    case 3: stress_residual32_p<3>(c, d_sigma_w, d_fe); break;
    default: stress_residual32_p<2>(c, d_sigma_w, d_fe); break;
    }
}

void launch_load_vector(ipfem_ctx *c)
{
    const int32_t neq = c->s.neq;
    const unsigned grid = (unsigned)std::max(1, std::min((neq + 255) / 256, 152 * 8));
    k_load_vector<<<grid, 256, 0, c->stream>>>(neq, c->load_factor, c->d_f0, c->d_df, c->d_lin);
}

// the instantiation for the mesh's colour count (at most kMaxColors, checked at setup)
template <class V, int NC = 0>
static void color_reduce_nc(ipfem_ctx *c, const V *d_fe, int with_load, double *d_res)
{
    if constexpr (NC <= kMaxColors) {
        const Setup &s = c->s;
        if (s.n_colors != NC) {
            color_reduce_nc<V, NC + 1>(c, d_fe, with_load, d_res);
            return;
        }
        const unsigned grid = (unsigned)((s.n_nodes + 255) / 256);
        k_color_reduce<V, NC><<<grid, 256, 0, c->stream>>>(s.n_nodes, c->d_inc, d_fe, with_load, c->d_lin,
                                                             c->d_fixed, d_res);
    }
}

void launch_color_reduce(ipfem_ctx *c, const double *d_fe, int with_load, double *d_res)
{
    color_reduce_nc<double>(c, d_fe, with_load, d_res);
}

void launch_color_reduce32(ipfem_ctx *c, const float *d_fe, int with_load, double *d_res)
{
    color_reduce_nc<float>(c, d_fe, with_load, d_res);
}

void launch_stiffness(ipfem_ctx *c)
{
    const Setup &s = c->s;
    cudaMemsetAsync(c->d_K, 0, (size_t)c->dsell.n_sell * 4 * sizeof(double), c->stream);
    for (int col = 0; col < s.n_colors; col++) {
        const int32_t first = s.color_ptr[col], n = s.color_ptr[col + 1] - first;
        if (n == 0) continue;
        const unsigned grid = (unsigned)((n + kStiffWarps - 1) / kStiffWarps);
        auto kern = s.order == 1 ? k_stiffness<double, 1> : (s.order == 3 ? k_stiffness<double, 3> :
                                                                            k_stiffness<double, 2>);
        kern<<<grid, kStiffWarps * 32, 0, c->stream>>>(n, c->d_color_els + first, s.n_ip, c->d_dphi, c->d_dep,
                                                       c->dsell.el_blk, c->d_K);
    }
    launch_jacobi(c);
}

void launch_jacobi(ipfem_ctx *c)
{
    const Setup &s = c->s;
    const unsigned g2 = (unsigned)((s.n_nodes + 255) / 256);
    if (c->precision == 1) {
        MixedBuffers &m = c->mx;
        k_jacobi<float><<<g2, 256, 0, c->stream>>>(s.n_nodes, fp32_layout(c).diag_blk, fp32_values(c), c->d_fixed,
                                                   m.dinv, m.binv);
    } else {
        k_jacobi<double><<<g2, 256, 0, c->stream>>>(s.n_nodes, c->dsell.diag_blk, c->d_K, c->d_fixed, c->d_dinv,
                                                    c->d_binv);
    }
}

void launch_stiffness32(ipfem_ctx *c)
{
    const Setup &s = c->s;
    const SellDev &L = fp32_layout(c);
    float *K = fp32_values(c);
    cudaMemsetAsync(K, 0, (size_t)L.n_sell * 4 * sizeof(float), c->stream);
    for (int col = 0; col < s.n_colors; col++) {
        const int32_t first = s.color_ptr[col], n = s.color_ptr[col + 1] - first;
        if (n == 0) continue;
        const unsigned grid = (unsigned)((n + kStiffWarps - 1) / kStiffWarps);
        auto kern = s.order == 1 ? k_stiffness<float, 1> : (s.order == 3 ? k_stiffness<float, 3> :
                                                                           k_stiffness<float, 2>);
        kern<<<grid, kStiffWarps * 32, 0, c->stream>>>(n, c->d_color_els + first, s.n_ip, c->mx.dphi, c->d_dep,
                                                       L.el_blk, K);
    }
    launch_jacobi(c);
}

}  // namespace ipfem
