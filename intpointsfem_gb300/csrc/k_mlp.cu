// Learned preconditioner: a per-node MLP (32 -> 128 -> 128 -> 2) applied inside
// flexible CG on the FP32 tangent.  No counterpart in the reference.
//
// Features of node i (structured node grid, neighbours outside the mesh read 0):
//   f[0..17]  residual of the 3x3 node patch (x, y), row by row, divided by
//             s_i = RMS of the patch residual
//   f[18..21] |r| of the four second-ring axial neighbours / s_i
//   f[22]     Dinv_x / Dinv_y of node i
//   f[23..26] Dinv_x(i) / Dinv_x(neighbour) for the four axial neighbours
//   f[27]     fraction of plastic integration points in the elements around i
//   f[28..29] grid coordinates a/(gr-1), b/(gt-1)
//   f[30..31] Dirichlet flags
// Output: z_i = (f[8..9] + W3^T h2 + b3) * s_i * Dinv_i.  With W3 = 0 the
// network is exactly Jacobi; training learns the correction on top of it.
//
// GEMMs run on the tensor cores in BF16 (operands rounded to BF16 in shared
// memory) with FP32 accumulation (mma.m16n8k16).
#include <cuda_bf16.h>

#include "ipfem_internal.h"

namespace ipfem {

constexpr unsigned FULLM = 0xffffffffu;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2])
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// ------------------------------------------------------------------ GEMM
// C[M][N] = alpha * op(A)[M][K] op(B)[K][N] (+ C if beta).  A and B are FP32 in
// global memory and rounded to BF16 when staged; FP32 accumulation.
//   transA = 0: A[m][k] = A[m*lda + k];   transA = 1: A[m][k] = A[k*lda + m]
//   transB = 0: B[k][n] = B[k*ldb + n];   transB = 1: B[k][n] = B[n*ldb + k]
// 64x64 tile per CTA, K step 32, 4 warps as 2 x 2, each warp 32 x 32.
constexpr int GT = 64, GK = 32, GPAD = 8;

__global__ void __launch_bounds__(128) k_gemm_bf16(int M, int N, int K, const float *__restrict__ A, int lda, int transA,
                                                   const float *__restrict__ B, int ldb, int transB,
                                                   float *__restrict__ C, int ldc, float alpha, int beta)
{
    __shared__ __align__(16) __nv_bfloat16 sA[GT][GK + GPAD];   // [m][k]
    __shared__ __align__(16) __nv_bfloat16 sB[GT][GK + GPAD];   // [n][k]
    const int m0 = blockIdx.y * GT, n0 = blockIdx.x * GT;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    const int g = lane >> 2, t = lane & 3;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int r = 0; r < 4; r++) acc[i][j][r] = 0.f;
    for (int k0 = 0; k0 < K; k0 += GK) {
        for (int e = threadIdx.x; e < GT * GK; e += 128) {
            int mm, kk;
            if (transA) { kk = e / GT; mm = e % GT; } else { mm = e / GK; kk = e % GK; }
            const int gm = m0 + mm, gk = k0 + kk;
            float v = 0.f;
            if (gm < M && gk < K) v = transA ? A[(size_t)gk * lda + gm] : A[(size_t)gm * lda + gk];
            sA[mm][kk] = __float2bfloat16_rn(v);
        }
        for (int e = threadIdx.x; e < GT * GK; e += 128) {
            int nn, kk;
            if (transB) { nn = e / GK; kk = e % GK; } else { kk = e / GT; nn = e % GT; }
            const int gn = n0 + nn, gk = k0 + kk;
            float v = 0.f;
            if (gn < N && gk < K) v = transB ? B[(size_t)gn * ldb + gk] : B[(size_t)gk * ldb + gn];
            sB[nn][kk] = __float2bfloat16_rn(v);
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < GK; ks += 16) {
            uint32_t af[2][4], bf[4][2];
#pragma unroll
            for (int i = 0; i < 2; i++) {
                const int r0 = wm + 16 * i + g;
                af[i][0] = *reinterpret_cast<const uint32_t *>(&sA[r0][ks + 2 * t]);
                af[i][1] = *reinterpret_cast<const uint32_t *>(&sA[r0 + 8][ks + 2 * t]);
                af[i][2] = *reinterpret_cast<const uint32_t *>(&sA[r0][ks + 8 + 2 * t]);
                af[i][3] = *reinterpret_cast<const uint32_t *>(&sA[r0 + 8][ks + 8 + 2 * t]);
            }
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int c0 = wn + 8 * j + g;
                bf[j][0] = *reinterpret_cast<const uint32_t *>(&sB[c0][ks + 2 * t]);
                bf[j][1] = *reinterpret_cast<const uint32_t *>(&sB[c0][ks + 8 + 2 * t]);
            }
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) mma_bf16(acc[i][j], af[i], bf[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const int gm = m0 + wm + 16 * i + g + ((r >> 1) << 3);
                const int gn = n0 + wn + 8 * j + 2 * t + (r & 1);
                if (gm < M && gn < N) {
                    float v = alpha * acc[i][j][r];
                    if (beta) v += C[(size_t)gm * ldc + gn];
                    C[(size_t)gm * ldc + gn] = v;
                }
            }
}

// ---------------------------------------------------- elementwise helpers
// H = relu(H + b) (b broadcast over rows of width n)
__global__ void k_bias_relu(int64_t rows, int n, float *__restrict__ H, const float *__restrict__ b, int relu)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= rows * n) return;
    float v = H[i] + b[i % n];
    H[i] = relu ? fmaxf(v, 0.f) : v;
}

// D = D * (H > 0)
__global__ void k_relu_mask(int64_t count, float *__restrict__ D, const float *__restrict__ H)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < count && !(H[i] > 0.f)) D[i] = 0.f;
}

// Output layer on CUDA cores: O[r][j] = X[r][8+j] + sum_n H2[r][n] W3[n][j] + b3[j]
__global__ void k_out_layer(int64_t rows, const float *__restrict__ X, const float *__restrict__ H2,
                            const float *__restrict__ W3, const float *__restrict__ b3, float *__restrict__ O)
{
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= rows) return;
    float o0 = 0.f, o1 = 0.f;
    for (int n = 0; n < 128; n++) {
        const float h = __bfloat162float(__float2bfloat16_rn(H2[r * 128 + n]));
        o0 = fmaf(h, __bfloat162float(__float2bfloat16_rn(W3[2 * n])), o0);
        o1 = fmaf(h, __bfloat162float(__float2bfloat16_rn(W3[2 * n + 1])), o1);
    }
    O[2 * r] = X[r * 32 + 8] + o0 + b3[0];
    O[2 * r + 1] = X[r * 32 + 9] + o1 + b3[1];
}

// loss = sum (O - Y)^2 / rows; dO = 2 (O - Y) / rows;  dH2 = dO W3^T (masked later)
__global__ void k_out_backward(int64_t rows, const float *__restrict__ O, const float *__restrict__ Y,
                               const float *__restrict__ W3, float *__restrict__ dO, float *__restrict__ dH2,
                               float *__restrict__ loss_part)
{
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    float l = 0.f;
    if (r < rows) {
        const float e0 = O[2 * r] - Y[2 * r], e1 = O[2 * r + 1] - Y[2 * r + 1];
        l = e0 * e0 + e1 * e1;
        const float s = 2.f / (float)rows;
        const float d0 = s * e0, d1 = s * e1;
        dO[2 * r] = d0;
        dO[2 * r + 1] = d1;
        for (int n = 0; n < 128; n++)
            dH2[r * 128 + n] = d0 * __bfloat162float(__float2bfloat16_rn(W3[2 * n])) +
                               d1 * __bfloat162float(__float2bfloat16_rn(W3[2 * n + 1]));
    }
    for (int off = 16; off; off >>= 1) l += __shfl_down_sync(FULLM, l, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss_part, l / (float)rows);
}

// column sums of D[rows][n] into g[n] (bias gradients); one thread per column
__global__ void k_colsum(int64_t rows, int n, const float *__restrict__ D, float *__restrict__ g)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    float s = 0.f;
    for (int64_t r = 0; r < rows; r++) s += D[r * n + c];
    g[c] = s;
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

// ------------------------------------------------------------ features
struct GridInfo {
    int32_t gr, gt;
};

__device__ __forceinline__ float2 rd_r(const float2 *__restrict__ r, GridInfo G, int a, int b)
{
    if (a < 0 || b < 0 || a >= G.gr || b >= G.gt) return make_float2(0.f, 0.f);
    return r[(int64_t)b * G.gr + a];
}

__device__ __forceinline__ float2 rd_d(const float2 *__restrict__ d, GridInfo G, int a, int b, bool &ok)
{
    ok = !(a < 0 || b < 0 || a >= G.gr || b >= G.gt);
    if (!ok) return make_float2(0.f, 0.f);
    return d[(int64_t)b * G.gr + a];
}

__device__ __forceinline__ float safe_ratio(float a, float b)
{
    return (a > 0.f && b > 0.f) ? a / b : 1.f;
}

// features of node i into f[32]; returns the scale s_i
__device__ __forceinline__ float node_features(int32_t i, GridInfo G, const float2 *__restrict__ r,
                                               const float2 *__restrict__ dinv, const float *__restrict__ pfrac,
                                               const uint8_t *__restrict__ fixed, float *f)
{
    const int a = i % G.gr, b = i / G.gr;
    float ss = 0.f;
    int k = 0;
#pragma unroll
    for (int db = -1; db <= 1; db++)
#pragma unroll
        for (int da = -1; da <= 1; da++) {
            const float2 v = rd_r(r, G, a + da, b + db);
            f[k++] = v.x;
            f[k++] = v.y;
            ss = fmaf(v.x, v.x, fmaf(v.y, v.y, ss));
        }
    const float s = sqrtf(ss / 9.f) + 1e-30f;
    const float inv = 1.f / s;
#pragma unroll
    for (int j = 0; j < 18; j++) f[j] *= inv;
    const int ra[4] = {-2, 2, 0, 0}, rb[4] = {0, 0, -2, 2};
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const float2 v = rd_r(r, G, a + ra[j], b + rb[j]);
        f[18 + j] = sqrtf(v.x * v.x + v.y * v.y) * inv;
    }
    bool ok;
    const float2 d0 = rd_d(dinv, G, a, b, ok);
    f[22] = safe_ratio(d0.x, d0.y);
    const int na[4] = {-1, 1, 0, 0}, nb[4] = {0, 0, -1, 1};
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const float2 dn = rd_d(dinv, G, a + na[j], b + nb[j], ok);
        f[23 + j] = ok ? safe_ratio(d0.x, dn.x) : 1.f;
    }
    f[27] = pfrac[i];
    f[28] = G.gr > 1 ? (float)a / (float)(G.gr - 1) : 0.f;
    f[29] = G.gt > 1 ? (float)b / (float)(G.gt - 1) : 0.f;
    f[30] = fixed[2 * (int64_t)i] ? 1.f : 0.f;
    f[31] = fixed[2 * (int64_t)i + 1] ? 1.f : 0.f;
    return s;
}

// features (rows of 32) and scales of all nodes, from an FP32 residual
__global__ void k_features(int32_t n_nodes, GridInfo G, const float *__restrict__ r, const float *__restrict__ dinv,
                           const float *__restrict__ pfrac, const uint8_t *__restrict__ fixed,
                           float *__restrict__ X, float *__restrict__ S)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_nodes) return;
    float f[32];
    const float s = node_features(i, G, reinterpret_cast<const float2 *>(r), reinterpret_cast<const float2 *>(dinv),
                                  pfrac, fixed, f);
#pragma unroll
    for (int j = 0; j < 32; j++) X[(int64_t)i * 32 + j] = f[j];
    S[i] = s;
}

// fraction of plastic points (committed m_type != 0) of the elements around each node
__global__ void k_plastic_fraction(int32_t n_el, const int32_t *__restrict__ dofs, const int8_t *__restrict__ mtype,
                                   float *__restrict__ num, float *__restrict__ den)
{
    const int32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_el) return;
    float p = 0.f;
    for (int q = 0; q < 9; q++) p += mtype[(int64_t)e * 9 + q] != 0 ? 1.f : 0.f;
    for (int n = 0; n < 9; n++) {
        const int32_t node = dofs[(int64_t)e * 18 + 2 * n] >> 1;
        atomicAdd(&num[node], p);
        atomicAdd(&den[node], 9.f);
    }
}

__global__ void k_ratio(int32_t n, float *__restrict__ num, const float *__restrict__ den)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) num[i] = den[i] > 0.f ? num[i] / den[i] : 0.f;
}

// ------------------------------------------------ fused preconditioner
// One CTA = 128 nodes, 8 warps; warp w owns rows 16w..16w+15.  Features ->
// smem (BF16), layer 1 and 2 on the tensor cores (FP32 accumulators in
// registers), layer 3 from the layer-2 accumulator fragments with a 4-lane
// shuffle reduction, then z = o * s * Dinv.  Also produces the partial dots
// r.z and r_old.z for the flexible-CG beta.
struct MlpDev {
    const __nv_bfloat16 *w1t;   // [128][32]  (n, k)
    const __nv_bfloat16 *w2t;   // [128][128] (n, k)
    const float *b1, *b2;       // [128]
    const float *w3;            // [128][2]
    const float *b3;            // [2]
};

constexpr int PT = 128;          // nodes per CTA

struct __align__(16) PrecSmem {
    __nv_bfloat16 x[PT][32 + 8];
    __nv_bfloat16 h[PT][128 + 8];
    __nv_bfloat16 w1[128][32 + 8];
    __nv_bfloat16 w2[128][128 + 8];
    float b1[128], b2[128], w3[128][2], b3[2];
    float own[PT][2];
    float sc[PT];
};

__device__ void mlp_tile(PrecSmem &S, int warp, int lane, float (&o)[2][2])
{
    const int g = lane >> 2, t = lane & 3;
    const int r0 = 16 * warp + g;
    float acc[16][4];
#pragma unroll
    for (int j = 0; j < 16; j++)
#pragma unroll
        for (int r = 0; r < 4; r++) acc[j][r] = 0.f;
    // layer 1: [16 x 32] x [32 x 128]
#pragma unroll
    for (int ks = 0; ks < 32; ks += 16) {
        uint32_t af[4];
        af[0] = *reinterpret_cast<const uint32_t *>(&S.x[r0][ks + 2 * t]);
        af[1] = *reinterpret_cast<const uint32_t *>(&S.x[r0 + 8][ks + 2 * t]);
        af[2] = *reinterpret_cast<const uint32_t *>(&S.x[r0][ks + 8 + 2 * t]);
        af[3] = *reinterpret_cast<const uint32_t *>(&S.x[r0 + 8][ks + 8 + 2 * t]);
#pragma unroll
        for (int j = 0; j < 16; j++) {
            uint32_t bf[2];
            bf[0] = *reinterpret_cast<const uint32_t *>(&S.w1[8 * j + g][ks + 2 * t]);
            bf[1] = *reinterpret_cast<const uint32_t *>(&S.w1[8 * j + g][ks + 8 + 2 * t]);
            mma_bf16(acc[j], af, bf);
        }
    }
    // bias + relu -> h (BF16), this warp's 16 rows only
#pragma unroll
    for (int j = 0; j < 16; j++) {
        const int c = 8 * j + 2 * t;
        const float v0 = fmaxf(acc[j][0] + S.b1[c], 0.f), v1 = fmaxf(acc[j][1] + S.b1[c + 1], 0.f);
        const float v2 = fmaxf(acc[j][2] + S.b1[c], 0.f), v3 = fmaxf(acc[j][3] + S.b1[c + 1], 0.f);
        *reinterpret_cast<uint32_t *>(&S.h[r0][c]) = pack_bf16(v0, v1);
        *reinterpret_cast<uint32_t *>(&S.h[r0 + 8][c]) = pack_bf16(v2, v3);
#pragma unroll
        for (int r = 0; r < 4; r++) acc[j][r] = 0.f;
    }
    __syncwarp();
    // layer 2: [16 x 128] x [128 x 128]
#pragma unroll
    for (int ks = 0; ks < 128; ks += 16) {
        uint32_t af[4];
        af[0] = *reinterpret_cast<const uint32_t *>(&S.h[r0][ks + 2 * t]);
        af[1] = *reinterpret_cast<const uint32_t *>(&S.h[r0 + 8][ks + 2 * t]);
        af[2] = *reinterpret_cast<const uint32_t *>(&S.h[r0][ks + 8 + 2 * t]);
        af[3] = *reinterpret_cast<const uint32_t *>(&S.h[r0 + 8][ks + 8 + 2 * t]);
#pragma unroll
        for (int j = 0; j < 16; j++) {
            uint32_t bf[2];
            bf[0] = *reinterpret_cast<const uint32_t *>(&S.w2[8 * j + g][ks + 2 * t]);
            bf[1] = *reinterpret_cast<const uint32_t *>(&S.w2[8 * j + g][ks + 8 + 2 * t]);
            mma_bf16(acc[j], af, bf);
        }
    }
    // layer 3 from the fragments: rows r0 (regs 0,1) and r0+8 (regs 2,3)
    float p00 = 0.f, p01 = 0.f, p10 = 0.f, p11 = 0.f;
#pragma unroll
    for (int j = 0; j < 16; j++) {
        const int c = 8 * j + 2 * t;
        const float h0 = __bfloat162float(__float2bfloat16_rn(fmaxf(acc[j][0] + S.b2[c], 0.f)));
        const float h1 = __bfloat162float(__float2bfloat16_rn(fmaxf(acc[j][1] + S.b2[c + 1], 0.f)));
        const float h2 = __bfloat162float(__float2bfloat16_rn(fmaxf(acc[j][2] + S.b2[c], 0.f)));
        const float h3 = __bfloat162float(__float2bfloat16_rn(fmaxf(acc[j][3] + S.b2[c + 1], 0.f)));
        p00 = fmaf(h0, S.w3[c][0], fmaf(h1, S.w3[c + 1][0], p00));
        p01 = fmaf(h0, S.w3[c][1], fmaf(h1, S.w3[c + 1][1], p01));
        p10 = fmaf(h2, S.w3[c][0], fmaf(h3, S.w3[c + 1][0], p10));
        p11 = fmaf(h2, S.w3[c][1], fmaf(h3, S.w3[c + 1][1], p11));
    }
#pragma unroll
    for (int off = 1; off <= 2; off <<= 1) {
        p00 += __shfl_xor_sync(FULLM, p00, off);
        p01 += __shfl_xor_sync(FULLM, p01, off);
        p10 += __shfl_xor_sync(FULLM, p10, off);
        p11 += __shfl_xor_sync(FULLM, p11, off);
    }
    o[0][0] = p00 + S.b3[0];
    o[0][1] = p01 + S.b3[1];
    o[1][0] = p10 + S.b3[0];
    o[1][1] = p11 + S.b3[1];
}

__device__ void load_weights(PrecSmem &S, const MlpDev &W)
{
    for (int e = threadIdx.x; e < 128 * 32; e += blockDim.x) S.w1[e / 32][e % 32] = W.w1t[e];
    for (int e = threadIdx.x; e < 128 * 128; e += blockDim.x) S.w2[e / 128][e % 128] = W.w2t[e];
    for (int e = threadIdx.x; e < 128; e += blockDim.x) {
        S.b1[e] = W.b1[e];
        S.b2[e] = W.b2[e];
        S.w3[e][0] = __bfloat162float(__float2bfloat16_rn(W.w3[2 * e]));
        S.w3[e][1] = __bfloat162float(__float2bfloat16_rn(W.w3[2 * e + 1]));
    }
    if (threadIdx.x < 2) S.b3[threadIdx.x] = W.b3[threadIdx.x];
}

// inference on given feature rows (testing / training evaluation): O[row][2]
__global__ void __launch_bounds__(256) k_mlp_infer_rows(int64_t rows, const float *__restrict__ X, MlpDev W,
                                                        float *__restrict__ O)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    PrecSmem &S = *reinterpret_cast<PrecSmem *>(smem_raw);
    load_weights(S, W);
    const int64_t base = (int64_t)blockIdx.x * PT;
    for (int e = threadIdx.x; e < PT * 32; e += blockDim.x) {
        const int row = e / 32, col = e % 32;
        const float v = (base + row < rows) ? X[(base + row) * 32 + col] : 0.f;
        S.x[row][col] = __float2bfloat16_rn(v);
        if (col == 8 || col == 9) S.own[row][col - 8] = v;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float o[2][2];
    mlp_tile(S, warp, lane, o);
    if ((lane & 3) == 0) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int row = 16 * warp + (lane >> 2) + 8 * h;
            if (base + row < rows) {
                O[2 * (base + row)] = S.own[row][0] + o[h][0];
                O[2 * (base + row) + 1] = S.own[row][1] + o[h][1];
            }
        }
    }
}

}  // namespace ipfem

namespace ipfem {

// ------------------------------------------------------ flexible CG (FP32)
// Reductions follow the tree of k_solver.cu (warp tree, 8-warp tree, last CTA).
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

// x = 0, p = 0, r = b*scale (FP64 -> FP32); b.b
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

// x += alpha p, r_old = r, r -= alpha q; r.r; convergence / stagnation
__global__ void __launch_bounds__(256) k_fcg_update(int32_t n_nodes, const float *__restrict__ p,
                                                    const float *__restrict__ q, float *__restrict__ x,
                                                    float *__restrict__ r, float *__restrict__ r_old, float *part,
                                                    int64_t n_part, unsigned *ticket, CGScalarsT<float> *sc,
                                                    int stall_window)
{
    if (*reinterpret_cast<volatile int *>(&sc->done)) return;
    const float alpha = *reinterpret_cast<volatile float *>(&sc->alpha);
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float v[1] = {0.f};
    if (i < n_nodes) {
        const float2 pp = reinterpret_cast<const float2 *>(p)[i];
        const float2 qq = reinterpret_cast<const float2 *>(q)[i];
        float2 xx = reinterpret_cast<float2 *>(x)[i];
        float2 rr = reinterpret_cast<float2 *>(r)[i];
        reinterpret_cast<float2 *>(r_old)[i] = rr;
        xx.x = fmaf(alpha, pp.x, xx.x);
        xx.y = fmaf(alpha, pp.y, xx.y);
        rr.x = fmaf(-alpha, qq.x, rr.x);
        rr.y = fmaf(-alpha, qq.y, rr.y);
        reinterpret_cast<float2 *>(x)[i] = xx;
        reinterpret_cast<float2 *>(r)[i] = rr;
        v[0] = fmaf(rr.y, rr.y, rr.x * rr.x);
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
            } else if (!(rr == rr) || sc->iters - sc->it_best > stall_window) {
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

// z = M(r) (fused features + MLP), partial r.z and r_old.z; last CTA:
// Polak-Ribiere beta = (r.z - r_old.z) / rz_prev (clipped at 0), rz = r.z.
// Persistent CTAs over 128-node tiles so the weights are staged once per CTA.
__global__ void __launch_bounds__(256) k_mlp_precond(int32_t n_nodes, GridInfo G, const float *__restrict__ r,
                                                     const float *__restrict__ r_old, const float *__restrict__ dinv,
                                                     const float *__restrict__ pfrac,
                                                     const uint8_t *__restrict__ fixed, MlpDev W,
                                                     float *__restrict__ z, float *part, int64_t n_part,
                                                     unsigned *ticket, CGScalarsT<float> *sc)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    PrecSmem &S = *reinterpret_cast<PrecSmem *>(smem_raw);
    if (*reinterpret_cast<volatile int *>(&sc->done)) return;
    load_weights(S, W);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t n_tiles = ((int64_t)n_nodes + PT - 1) / PT;
    float vz = 0.f, vc = 0.f;
    const float2 *r2 = reinterpret_cast<const float2 *>(r);
    const float2 *ro2 = reinterpret_cast<const float2 *>(r_old);
    const float2 *d2 = reinterpret_cast<const float2 *>(dinv);
    for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const int64_t base = tile * PT;
        __syncthreads();   // weights staged / previous tile finished with S.x, S.h
        if (threadIdx.x < PT) {
            const int64_t node = base + threadIdx.x;
            float f[32];
            float s = 1.f;
            if (node < n_nodes) {
                s = node_features((int32_t)node, G, r2, d2, pfrac, fixed, f);
            } else {
#pragma unroll
                for (int j = 0; j < 32; j++) f[j] = 0.f;
            }
#pragma unroll
            for (int j = 0; j < 32; j += 2)
                *reinterpret_cast<uint32_t *>(&S.x[threadIdx.x][j]) = pack_bf16(f[j], f[j + 1]);
            S.own[threadIdx.x][0] = f[8];
            S.own[threadIdx.x][1] = f[9];
            S.sc[threadIdx.x] = s;
        }
        __syncthreads();
        float o[2][2];
        mlp_tile(S, warp, lane, o);
        if ((lane & 3) == 0) {
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int row = 16 * warp + (lane >> 2) + 8 * h;
                const int64_t node = base + row;
                if (node < n_nodes) {
                    const float2 di = d2[node];
                    const float s = S.sc[row];
                    float2 zz;
                    zz.x = (S.own[row][0] + o[h][0]) * s * di.x;
                    zz.y = (S.own[row][1] + o[h][1]) * s * di.y;
                    reinterpret_cast<float2 *>(z)[node] = zz;
                    const float2 rr = r2[node], ro = ro2[node];
                    vz = fmaf(rr.y, zz.y, fmaf(rr.x, zz.x, vz));
                    vc = fmaf(ro.y, zz.y, fmaf(ro.x, zz.x, vc));
                }
            }
        }
    }
    float v[2] = {vz, vc};
    if (fcg_partials<2>(v, part, n_part, ticket)) {
        float out[2];
        fcg_final<2>(part, n_part, out);
        if (threadIdx.x == 0) {
            const float rz = out[0], cross = out[1];
            float beta = (sc->rz > 0.f) ? (rz - cross) / sc->rz : 0.f;
            if (!(beta > 0.f)) beta = 0.f;
            sc->beta = beta;
            sc->rz = rz;
            if (!(rz > 0.f)) {          // the learned step is not a descent direction
                sc->done = 1;
                sc->status = kStatusFallback;
            }
            *ticket = 0u;
        }
    }
}

// ---------------------------------------------------------------- host side

static MlpDev mlp_dev(ipfem_ctx *c)
{
    MlpBuffers &m = c->mlp;
    MlpDev W;
    W.w1t = static_cast<const __nv_bfloat16 *>(m.w1t);
    W.w2t = static_cast<const __nv_bfloat16 *>(m.w2t);
    W.b1 = m.params + kOffB1;
    W.b2 = m.params + kOffB2;
    W.w3 = m.params + kOffW3;
    W.b3 = m.params + kOffB3;
    return W;
}

// BF16 copies of W1, W2 in the (n, k) layout of the tensor-core B operand
__global__ void k_pack_w(const float *__restrict__ P, __nv_bfloat16 *__restrict__ w1t, __nv_bfloat16 *__restrict__ w2t)
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
}

void mlp_pack_weights(ipfem_ctx *c)
{
    k_pack_w<<<64, 256, 0, c->stream>>>(c->mlp.params, static_cast<__nv_bfloat16 *>(c->mlp.w1t),
                                        static_cast<__nv_bfloat16 *>(c->mlp.w2t));
}

void launch_plastic_fraction(ipfem_ctx *c)
{
    const Setup &s = c->s;
    cudaMemsetAsync(c->mlp.pfrac, 0, (size_t)s.n_nodes * sizeof(float), c->stream);
    cudaMemsetAsync(c->mlp.pden, 0, (size_t)s.n_nodes * sizeof(float), c->stream);
    k_plastic_fraction<<<(s.n_el + 255) / 256, 256, 0, c->stream>>>(s.n_el, c->d_dofs, c->d_mtype, c->mlp.pfrac,
                                                                    c->mlp.pden);
    k_ratio<<<(s.n_nodes + 255) / 256, 256, 0, c->stream>>>(s.n_nodes, c->mlp.pfrac, c->mlp.pden);
}

void launch_features(ipfem_ctx *c, const float *d_r, float *d_X, float *d_S)
{
    GridInfo G{c->mlp.gr, c->mlp.gt};
    k_features<<<(c->s.n_nodes + 127) / 128, 128, 0, c->stream>>>(c->s.n_nodes, G, d_r, c->mx.dinv, c->mlp.pfrac,
                                                                  c->d_fixed, d_X, d_S);
}

// opt-in to the shared memory the fused kernels need (once, outside any capture)
cudaError_t mlp_configure()
{
    const int sm = (int)sizeof(PrecSmem);
    cudaError_t e = cudaFuncSetAttribute(k_mlp_infer_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_mlp_precond, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
}

void launch_mlp_infer_rows(ipfem_ctx *c, int64_t rows, const float *d_X, float *d_O)
{
    const size_t sm = sizeof(PrecSmem);
    k_mlp_infer_rows<<<(unsigned)((rows + PT - 1) / PT), 256, sm, c->stream>>>(rows, d_X, mlp_dev(c), d_O);
}

static unsigned fcg_grid(const ipfem_ctx *c)
{
    return (unsigned)((c->s.n_nodes + 255) / 256);
}

static unsigned precond_grid(const ipfem_ctx *c)
{
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    const int64_t tiles = ((int64_t)c->s.n_nodes + PT - 1) / PT;
    return (unsigned)std::min<int64_t>(tiles, 2 * (int64_t)sms);
}

static void launch_precond(ipfem_ctx *c)
{
    const size_t sm = sizeof(PrecSmem);
    GridInfo G{c->mlp.gr, c->mlp.gt};
    MixedBuffers &m = c->mx;
    // the precond partials use the third slot of the FP64 partial array (as floats)
    float *part = reinterpret_cast<float *>(c->d_part);
    k_mlp_precond<<<precond_grid(c), 256, sm, c->stream>>>(c->s.n_nodes, G, m.r, c->mlp.r_old, m.dinv,
                                                          c->mlp.pfrac, c->d_fixed, mlp_dev(c), m.z, part,
                                                          precond_grid(c), c->d_counters + 7, m.sc);
}

void launch_fcg_init(ipfem_ctx *c, const double *d_b, double scale, float rtol, int max_it)
{
    MixedBuffers &m = c->mx;
    k_fcg_init<<<fcg_grid(c), 256, 0, c->stream>>>(c->s.n_nodes, d_b, scale, m.x, m.r, m.p, c->mlp.r_old, m.part,
                                                   (int64_t)fcg_grid(c), c->d_counters + 4, m.sc, rtol, max_it);
    launch_precond(c);
    launch_cg32_pupdate_only(c);
}

void launch_fcg_iteration(ipfem_ctx *c)
{
    MixedBuffers &m = c->mx;
    launch_cg32_spmv_only(c);
    k_fcg_update<<<fcg_grid(c), 256, 0, c->stream>>>(c->s.n_nodes, m.p, m.q, m.x, m.r, c->mlp.r_old, m.part,
                                                     (int64_t)fcg_grid(c), c->d_counters + 6, m.sc, 400);
    launch_precond(c);
    launch_cg32_pupdate_only(c);
}

// One forward (and backward + Adam step if update) over `rows` training rows.
void mlp_train_step(ipfem_ctx *c, int64_t rows, const float *X, const float *Y, float *H1, float *H2, float *O,
                    float *dO, float *dH1, float *dH2, bool update, float lr)
{
    MlpBuffers &m = c->mlp;
    cudaStream_t st = c->stream;
    const int R = (int)rows;
    auto gemm = [&](int M, int N, int K, const float *A, int lda, int tA, const float *B, int ldb, int tB, float *C_,
                    int ldc) {
        dim3 grid((N + GT - 1) / GT, (M + GT - 1) / GT);
        k_gemm_bf16<<<grid, 128, 0, st>>>(M, N, K, A, lda, tA, B, ldb, tB, C_, ldc, 1.f, 0);
    };
    const unsigned eb = (unsigned)((rows * 128 + 255) / 256);
    // forward
    gemm(R, 128, 32, X, 32, 0, m.params + kOffW1, 128, 0, H1, 128);
    k_bias_relu<<<eb, 256, 0, st>>>(rows, 128, H1, m.params + kOffB1, 1);
    gemm(R, 128, 128, H1, 128, 0, m.params + kOffW2, 128, 0, H2, 128);
    k_bias_relu<<<eb, 256, 0, st>>>(rows, 128, H2, m.params + kOffB2, 1);
    const unsigned rb = (unsigned)((rows + 255) / 256);
    k_out_layer<<<rb, 256, 0, st>>>(rows, X, H2, m.params + kOffW3, m.params + kOffB3, O);
    // backward
    cudaMemsetAsync(m.loss, 0, sizeof(float), st);
    k_out_backward<<<rb, 256, 0, st>>>(rows, O, Y, m.params + kOffW3, dO, dH2, m.loss);
    k_relu_mask<<<eb, 256, 0, st>>>(rows * 128, dH2, H2);
    gemm(128, 2, R, H2, 128, 1, dO, 2, 0, m.grads + kOffW3, 2);            // dW3 = H2^T dO
    k_colsum<<<1, 32, 0, st>>>(rows, 2, dO, m.grads + kOffB3);
    gemm(128, 128, R, H1, 128, 1, dH2, 128, 0, m.grads + kOffW2, 128);     // dW2 = H1^T dH2
    k_colsum<<<1, 128, 0, st>>>(rows, 128, dH2, m.grads + kOffB2);
    gemm(R, 128, 128, dH2, 128, 0, m.params + kOffW2, 128, 1, dH1, 128);   // dH1 = dH2 W2^T
    k_relu_mask<<<eb, 256, 0, st>>>(rows * 128, dH1, H1);
    gemm(32, 128, R, X, 32, 1, dH1, 128, 0, m.grads + kOffW1, 128);        // dW1 = X^T dH1
    k_colsum<<<1, 128, 0, st>>>(rows, 128, dH1, m.grads + kOffB1);
    if (update) {
        m.adam_t += 1;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f - powf(b1, (float)m.adam_t), c2 = 1.f - powf(b2, (float)m.adam_t);
        k_adam<<<(kMlpParams + 255) / 256, 256, 0, st>>>(kMlpParams, m.params, m.grads, m.m, m.v, lr, b1, b2, 1e-8f,
                                                         c1, c2);
        mlp_pack_weights(c);
    }
}

}  // namespace ipfem
