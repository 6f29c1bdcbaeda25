// Fused per-node network (32 -> 128 -> 128 -> 20) on the 5th-generation tensor
// cores: tcgen05.mma (kind::f16, BF16 operands from shared memory, FP32
// accumulators in tensor memory), tcgen05.ld for the epilogues.  Tiles of 128
// nodes; node row r is TMEM lane r.  Layer 1 accumulates in TMEM columns
// 0..127, layer 2 in 128..255, layer 3 (N padded to 32) reuses columns 0..31.
// The inference kernel runs 8 warps per CTA: warps w and w + 4 read the
// same lane quadrant (a warp may only access lanes 32 (w % 4) .. + 31) and
// split the columns, so each epilogue takes half as long; the training
// kernels run 4 warps, thread t = row t.
//
// Shared-memory operands use the canonical K-major layout without swizzle:
// core matrices of 8 rows x 16 bytes (8 BF16 along K) stored as 128
// contiguous bytes; the 8-row groups of one K chunk follow each other (stride
// SBO = 128 B), and the K chunks follow at stride LBO = rows * 16 B.
#include <cuda_bf16.h>

#include "ipfem_internal.h"
#include "tma.cuh"

namespace ipfem {

namespace {

constexpr int TC_ROWS = 128;          // nodes per tile (MMA M)
constexpr int TC_NOUT = 20, TC_N3 = 32;
constexpr uint32_t TC_TMEM_COLS = 256;

// byte offsets of the operands inside the dynamic shared memory
constexpr uint32_t OFF_X = 0;                        // 128 x 32  : 8 KB
constexpr uint32_t OFF_W1 = OFF_X + 128 * 32 * 2;    // 128 x 32  : 8 KB
constexpr uint32_t OFF_H = OFF_W1 + 128 * 32 * 2;    // 128 x 128 : 32 KB
constexpr uint32_t OFF_W2 = OFF_H + 128 * 128 * 2;   // 128 x 128 : 32 KB
constexpr uint32_t OFF_W3 = OFF_W2 + 128 * 128 * 2;  // 32 x 128  : 8 KB
constexpr uint32_t OFF_B1 = OFF_W3 + 32 * 128 * 2;   // 128 floats
constexpr uint32_t OFF_B2 = OFF_B1 + 512;
constexpr uint32_t OFF_B3 = OFF_B2 + 512;            // 32 floats
constexpr uint32_t OFF_BAR = OFF_B3 + 128;           // mbarrier
constexpr uint32_t OFF_TMEM = OFF_BAR + 8;           // TMEM base written by tcgen05.alloc
constexpr uint32_t TC_SMEM = OFF_TMEM + 8;

// canonical offset of element (r, k) of an operand with `rows` rows
__device__ __forceinline__ uint32_t cano(uint32_t r, uint32_t k, uint32_t rows)
{
    return (k >> 3) * (rows * 16u) + (r >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// shared-memory matrix descriptor (tcgen05): start, LBO, SBO, version 1, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor: D FP32, A and B BF16, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t m, uint32_t n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before()
{
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after()
{
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void fence_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr)
                 : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pk_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

// all threads wait for the barrier phase (bounded); uniform result
__device__ __forceinline__ bool wait_all(uint64_t *bar, uint32_t phase)
{
    const bool ok = mbar_wait_bounded(bar, phase);
    return __syncthreads_and(ok ? 1 : 0) != 0;
}

// relu(v + b) of 32 columns starting at column c0 as BF16 into H (row r)
__device__ __forceinline__ void store_hidden(unsigned char *smem, uint32_t r, uint32_t c0, const float (&v)[32],
                                             const float *b)
{
#pragma unroll
    for (int q = 0; q < 4; q++) {
        uint4 w;
        w.x = pk_bf16(fmaxf(v[8 * q + 0] + b[c0 + 8 * q + 0], 0.f), fmaxf(v[8 * q + 1] + b[c0 + 8 * q + 1], 0.f));
        w.y = pk_bf16(fmaxf(v[8 * q + 2] + b[c0 + 8 * q + 2], 0.f), fmaxf(v[8 * q + 3] + b[c0 + 8 * q + 3], 0.f));
        w.z = pk_bf16(fmaxf(v[8 * q + 4] + b[c0 + 8 * q + 4], 0.f), fmaxf(v[8 * q + 5] + b[c0 + 8 * q + 5], 0.f));
        w.w = pk_bf16(fmaxf(v[8 * q + 6] + b[c0 + 8 * q + 6], 0.f), fmaxf(v[8 * q + 7] + b[c0 + 8 * q + 7], 0.f));
        *reinterpret_cast<uint4 *>(smem + OFF_H + cano(r, c0 + 8 * q, 128)) = w;
    }
}

// the same 32 hidden values in FP32 to row r of a [rows][128] array
__device__ __forceinline__ void store_hidden_f32(float *__restrict__ Hrow, uint32_t c0, const float (&v)[32],
                                                 const float *b)
{
#pragma unroll
    for (int q = 0; q < 8; q++)
        reinterpret_cast<float4 *>(Hrow + c0)[q] =
            make_float4(fmaxf(v[4 * q + 0] + b[c0 + 4 * q + 0], 0.f), fmaxf(v[4 * q + 1] + b[c0 + 4 * q + 1], 0.f),
                        fmaxf(v[4 * q + 2] + b[c0 + 4 * q + 2], 0.f), fmaxf(v[4 * q + 3] + b[c0 + 4 * q + 3], 0.f));
}

}  // namespace

// O[rows][20] = network(X[rows][32]); persistent CTAs of kNetThreads = 256
// threads over 128-row tiles: thread t owns row t % 128 and, of every
// 128-column epilogue, the columns 64 (t / 128) .. + 63.  With H1 and H2
// given, the hidden layers relu(X W1 + b1) and relu(H1 W2 + b2) are also
// written out in FP32 ([rows][128] each; the BF16 operand of the next layer is
// the same value rounded), for the training backward.  A barrier wait that
// runs out sets *err = 3 and the CTA stops.
constexpr int kNetThreads = 256;

__global__ void __launch_bounds__(kNetThreads) k_patch_net_tc(int64_t rows, const float *__restrict__ X,
                                                              const __nv_bfloat16 *__restrict__ w1t,
                                                              const __nv_bfloat16 *__restrict__ w2t,
                                                              const __nv_bfloat16 *__restrict__ w3t,
                                                              const float *__restrict__ b1,
                                                              const float *__restrict__ b2,
                                                              const float *__restrict__ b3, float *__restrict__ O,
                                                              float *__restrict__ H1, float *__restrict__ H2,
                                                              int *err)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    const uint32_t r = tid & 127u, half = tid >> 7;                 // row of the tile, column half
    const uint32_t sbase = smem_u32(smem);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + OFF_BAR);
    // weights and biases into the canonical layouts (16 bytes = 8 BF16 along K per copy)
    for (uint32_t e = tid; e < 128 * 4; e += blockDim.x) {          // W1^T: 128 x 32
        const uint32_t n = e >> 2, q = e & 3;
        *reinterpret_cast<uint4 *>(smem + OFF_W1 + cano(n, 8 * q, 128)) =
            *reinterpret_cast<const uint4 *>(w1t + n * 32 + 8 * q);
    }
    for (uint32_t e = tid; e < 128 * 16; e += blockDim.x) {         // W2^T: 128 x 128
        const uint32_t n = e >> 4, q = e & 15;
        *reinterpret_cast<uint4 *>(smem + OFF_W2 + cano(n, 8 * q, 128)) =
            *reinterpret_cast<const uint4 *>(w2t + n * 128 + 8 * q);
    }
    for (uint32_t e = tid; e < TC_N3 * 16; e += blockDim.x) {       // W3^T: 32 x 128 (rows >= 24 zero)
        const uint32_t n = e >> 4, q = e & 15;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (n < 24) v = *reinterpret_cast<const uint4 *>(w3t + n * 128 + 8 * q);
        *reinterpret_cast<uint4 *>(smem + OFF_W3 + cano(n, 8 * q, TC_N3)) = v;
    }
    float *sb1 = reinterpret_cast<float *>(smem + OFF_B1), *sb2 = reinterpret_cast<float *>(smem + OFF_B2);
    float *sb3 = reinterpret_cast<float *>(smem + OFF_B3);
    if (tid < 128) {
        sb1[tid] = b1[tid];
        sb2[tid] = b2[tid];
    }
    if (tid < TC_N3) sb3[tid] = tid < TC_NOUT ? b3[tid] : 0.f;
    if (tid == 0) mbar_init(bar, 1);
    // tensor memory: one warp allocates 256 columns
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sbase + OFF_TMEM),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(smem + OFF_TMEM);
    const uint32_t lane_t = tmem + (((warp & 3u) * 32u) << 16);      // this warp's TMEM lanes
    const uint32_t c_lo = 64u * half;                                 // this thread's first epilogue column
    constexpr uint32_t ID128 = idesc_bf16(128, 128), ID32 = idesc_bf16(128, TC_N3);
    uint32_t phase = 0;
    bool ok = true;
    const int64_t n_tiles = (rows + TC_ROWS - 1) / TC_ROWS;
    // this thread's 16 features of its row in the CTA's next tile, loaded one
    // tile ahead so that the load latency overlaps the current tile's layers
    float4 f[4];
    auto load_features = [&](int64_t tile) {
        const int64_t row = tile * TC_ROWS + r;
#pragma unroll
        for (int j = 0; j < 4; j++)
            f[j] = (tile < n_tiles && row < rows)
                       ? __ldcs(reinterpret_cast<const float4 *>(X + row * 32 + 16 * half) + j)
                       : make_float4(0.f, 0.f, 0.f, 0.f);
    };
    load_features(blockIdx.x);
    for (int64_t tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
        const int64_t row = tile * TC_ROWS + r;
        // features -> BF16 A operand, then the next tile's features in flight
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const uint4 w = make_uint4(pk_bf16(f[2 * q].x, f[2 * q].y), pk_bf16(f[2 * q].z, f[2 * q].w),
                                       pk_bf16(f[2 * q + 1].x, f[2 * q + 1].y), pk_bf16(f[2 * q + 1].z, f[2 * q + 1].w));
            *reinterpret_cast<uint4 *>(smem + OFF_X + cano(r, 16 * half + 8 * q, 128)) = w;
        }
        load_features(tile + gridDim.x);
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        // layer 1: D[0..127] = X W1 (K = 32: two K-steps of 16)
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (uint32_t kk = 0; kk < 2; kk++)
                tc_mma(tmem, sdesc(sbase + OFF_X + kk * 2 * 2048, 2048, 128),
                       sdesc(sbase + OFF_W1 + kk * 2 * 2048, 2048, 128), ID128, kk);
            tc_commit(sbase + OFF_BAR);
        }
        ok = wait_all(bar, phase);
        phase ^= 1u;
        if (!ok) break;
        tc_fence_after();
#pragma unroll 1
        for (uint32_t c = c_lo; c < c_lo + 64; c += 32) {
            float v[32];
            tc_ld32(lane_t + c, v);
            store_hidden(smem, r, c, v, sb1);
            if (H1 && row < rows) store_hidden_f32(H1 + row * 128, c, v, sb1);
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        // layer 2: D[128..255] = H1 W2 (K = 128)
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (uint32_t kk = 0; kk < 8; kk++)
                tc_mma(tmem + 128, sdesc(sbase + OFF_H + kk * 2 * 2048, 2048, 128),
                       sdesc(sbase + OFF_W2 + kk * 2 * 2048, 2048, 128), ID128, kk);
            tc_commit(sbase + OFF_BAR);
        }
        ok = wait_all(bar, phase);
        phase ^= 1u;
        if (!ok) break;
        tc_fence_after();
#pragma unroll 1
        for (uint32_t c = c_lo; c < c_lo + 64; c += 32) {
            float v[32];
            tc_ld32(lane_t + 128 + c, v);
            store_hidden(smem, r, c, v, sb2);
            if (H2 && row < rows) store_hidden_f32(H2 + row * 128, c, v, sb2);
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        // layer 3: D[0..31] = H2 W3 (N = 32, K = 128)
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (uint32_t kk = 0; kk < 8; kk++)
                tc_mma(tmem, sdesc(sbase + OFF_H + kk * 2 * 2048, 2048, 128),
                       sdesc(sbase + OFF_W3 + kk * 2 * 512, 512, 128), ID32, kk);
            tc_commit(sbase + OFF_BAR);
        }
        ok = wait_all(bar, phase);
        phase ^= 1u;
        if (!ok) break;
        tc_fence_after();
        if (half == 0) {
            float v[32];
            tc_ld32(lane_t, v);
            if (row < rows) {
                float4 *o = reinterpret_cast<float4 *>(O + row * TC_NOUT);
#pragma unroll
                for (int j = 0; j < 5; j++)
                    o[j] = make_float4(v[4 * j] + sb3[4 * j], v[4 * j + 1] + sb3[4 * j + 1],
                                       v[4 * j + 2] + sb3[4 * j + 2], v[4 * j + 3] + sb3[4 * j + 3]);
            }
        }
        tc_fence_before();
        __syncthreads();
    }
    if (!ok && tid == 0) atomicExch(err, 3);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS)
                     : "memory");
}

// Backward of the two hidden layers for the training pass, per 128-row tile:
//   dH2 = (dO W3^T) * (H2 > 0)     (K = 20, padded to 32)
//   dH1 = (dH2 W2^T) * (H1 > 0)    (K = 128)
// dO [rows][20], H1, H2, dH1, dH2 [rows][128], all FP32; W = the FP32
// parameter vector (W2 [128][128] at kOffW2, W3 [128][20] at kOffW3,
// row-major), rounded to BF16 once per CTA into the B operands.  dH2 is kept
// on chip as the BF16 A operand of the second product.  Persistent CTAs of
// 128 threads (thread t = row t = TMEM lane t), one 128-column accumulator
// used by both products; the mask rows of H2 and H1 are loaded while the MMAs
// run.  Shared-memory regions: OFF_X = dO tile (128 x 32), OFF_W1 = W3 as
// N = 128 x K = 32, OFF_H = dH2 tile, OFF_W2 = W2 as N = 128 x K = 128.
__global__ void __launch_bounds__(128) k_patch_net_bwd_tc(int64_t rows, const float *__restrict__ dO,
                                                          const float *__restrict__ H1,
                                                          const float *__restrict__ H2,
                                                          const float *__restrict__ W, float *__restrict__ dH2,
                                                          float *__restrict__ dH1, int *err)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    const uint32_t sbase = smem_u32(smem);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + OFF_BAR);
    // B(n = j, k = o) = W3[j][o] (o < 20), 8 K values per 16-byte store
    for (uint32_t e = tid; e < 128 * 4; e += blockDim.x) {
        const uint32_t n = e >> 2, q = e & 3;
        float f[8];
#pragma unroll
        for (int j = 0; j < 8; j++) f[j] = (8 * q + j < 20) ? W[kOffW3 + n * 20 + 8 * q + j] : 0.f;
        *reinterpret_cast<uint4 *>(smem + OFF_W1 + cano(n, 8 * q, 128)) =
            make_uint4(pk_bf16(f[0], f[1]), pk_bf16(f[2], f[3]), pk_bf16(f[4], f[5]), pk_bf16(f[6], f[7]));
    }
    // B(n = i, k = j) = W2[i][j]
    for (uint32_t e = tid; e < 128 * 16; e += blockDim.x) {
        const uint32_t n = e >> 4, q = e & 15;
        const float4 f0 = *reinterpret_cast<const float4 *>(W + kOffW2 + n * 128 + 8 * q);
        const float4 f1 = *reinterpret_cast<const float4 *>(W + kOffW2 + n * 128 + 8 * q + 4);
        *reinterpret_cast<uint4 *>(smem + OFF_W2 + cano(n, 8 * q, 128)) =
            make_uint4(pk_bf16(f0.x, f0.y), pk_bf16(f0.z, f0.w), pk_bf16(f1.x, f1.y), pk_bf16(f1.z, f1.w));
    }
    if (tid == 0) mbar_init(bar, 1);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sbase + OFF_TMEM),
                     "r"(128u)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(smem + OFF_TMEM);
    const uint32_t lane_t = tmem + ((warp * 32u) << 16);
    constexpr uint32_t ID128 = idesc_bf16(128, 128);
    uint32_t phase = 0;
    bool ok = true;
    const int64_t n_tiles = (rows + TC_ROWS - 1) / TC_ROWS;
    for (int64_t tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
        const int64_t row = tile * TC_ROWS + tid;
        const bool live = row < rows;
        {
            float f[32];
#pragma unroll
            for (int j = 0; j < 5; j++) {
                const float4 t = live ? reinterpret_cast<const float4 *>(dO + row * 20)[j] : make_float4(0.f, 0.f, 0.f, 0.f);
                f[4 * j] = t.x; f[4 * j + 1] = t.y; f[4 * j + 2] = t.z; f[4 * j + 3] = t.w;
            }
#pragma unroll
            for (int j = 20; j < 32; j++) f[j] = 0.f;
#pragma unroll
            for (int q = 0; q < 4; q++)
                *reinterpret_cast<uint4 *>(smem + OFF_X + cano(tid, 8 * q, 128)) =
                    make_uint4(pk_bf16(f[8 * q], f[8 * q + 1]), pk_bf16(f[8 * q + 2], f[8 * q + 3]),
                               pk_bf16(f[8 * q + 4], f[8 * q + 5]), pk_bf16(f[8 * q + 6], f[8 * q + 7]));
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (uint32_t kk = 0; kk < 2; kk++)
                tc_mma(tmem, sdesc(sbase + OFF_X + kk * 2 * 2048, 2048, 128),
                       sdesc(sbase + OFF_W1 + kk * 2 * 2048, 2048, 128), ID128, kk);
            tc_commit(sbase + OFF_BAR);
        }
        float4 hm[32];                               // mask row, loaded while the MMAs run
#pragma unroll
        for (int j = 0; j < 32; j++)
            hm[j] = live ? reinterpret_cast<const float4 *>(H2 + row * 128)[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        ok = wait_all(bar, phase);
        phase ^= 1u;
        if (!ok) break;
        tc_fence_after();
#pragma unroll
        for (uint32_t c = 0; c < 4; c++) {
            float v[32];
            tc_ld32(lane_t + 32 * c, v);
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const float4 m = hm[8 * c + q];
                if (!(m.x > 0.f)) v[4 * q] = 0.f;
                if (!(m.y > 0.f)) v[4 * q + 1] = 0.f;
                if (!(m.z > 0.f)) v[4 * q + 2] = 0.f;
                if (!(m.w > 0.f)) v[4 * q + 3] = 0.f;
                if (live)
                    reinterpret_cast<float4 *>(dH2 + row * 128 + 32 * c)[q] =
                        make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            }
#pragma unroll
            for (int q = 0; q < 4; q++)
                *reinterpret_cast<uint4 *>(smem + OFF_H + cano(tid, 32 * c + 8 * q, 128)) =
                    make_uint4(pk_bf16(v[8 * q], v[8 * q + 1]), pk_bf16(v[8 * q + 2], v[8 * q + 3]),
                               pk_bf16(v[8 * q + 4], v[8 * q + 5]), pk_bf16(v[8 * q + 6], v[8 * q + 7]));
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (uint32_t kk = 0; kk < 8; kk++)
                tc_mma(tmem, sdesc(sbase + OFF_H + kk * 2 * 2048, 2048, 128),
                       sdesc(sbase + OFF_W2 + kk * 2 * 2048, 2048, 128), ID128, kk);
            tc_commit(sbase + OFF_BAR);
        }
#pragma unroll
        for (int j = 0; j < 32; j++)
            hm[j] = live ? reinterpret_cast<const float4 *>(H1 + row * 128)[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        ok = wait_all(bar, phase);
        phase ^= 1u;
        if (!ok) break;
        tc_fence_after();
#pragma unroll
        for (uint32_t c = 0; c < 4; c++) {
            float v[32];
            tc_ld32(lane_t + 32 * c, v);
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const float4 m = hm[8 * c + q];
                if (live)
                    reinterpret_cast<float4 *>(dH1 + row * 128 + 32 * c)[q] =
                        make_float4(m.x > 0.f ? v[4 * q] : 0.f, m.y > 0.f ? v[4 * q + 1] : 0.f,
                                    m.z > 0.f ? v[4 * q + 2] : 0.f, m.w > 0.f ? v[4 * q + 3] : 0.f);
            }
        }
        tc_fence_before();
        __syncthreads();
    }
    if (!ok && tid == 0) atomicExch(err, 3);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128u) : "memory");
}

// ------------------------------------------------ general GEMM on tcgen05
// C[M][N] = op(A)[M][K] op(B)[K][N] for the weight gradients of the training
// pass: A and B FP32 in global memory, rounded to BF16 while they are staged
// into the canonical K-major layouts, FP32 accumulators in tensor memory.
//   transA = 0: A[m][k] = A[m*lda + k];   transA = 1: A[m][k] = A[k*lda + m]
//   transB = 0: B[k][n] = B[k*ldb + n];   transB = 1: B[k][n] = B[n*ldb + k]
// With colsum given (B read with transB = 0, N <= 128), the CTAs of the first
// M tile also write the FP32 column sums of B over their K range to
// colsum[z*N + n] (the bias gradient of a weight-gradient GEMM).
// One CTA of 128 threads per 128 x 128 tile of C (TMEM lane t = row m0 + t);
// K in chunks of 32 (two MMAs of K = 16).  Thread t stages row t of both
// operand tiles: 32 FP32 loads into registers (float4 along a contiguous K,
// else one coalesced load per K across the warp), then four 16-byte stores
// of 8 BF16 each, which fall on consecutive 16-byte slots across the warp.
// The loads of chunk i+1 are issued while the MMAs of chunk i run.  Split K:
// CTA z covers k in [z*kchunk, (z+1)*kchunk) (kchunk a multiple of 32) and
// writes C + z*M*ldc.  The dynamic shared-memory request keeps at most 4 CTAs
// on an SM, so that their 128 TMEM columns each always fit and tcgen05.alloc
// never waits.
namespace {
constexpr uint32_t G_OFF_A = 0;                  // 128 x 32 BF16: 8 KB
constexpr uint32_t G_OFF_B = 128 * 32 * 2;       // 128 x 32 BF16: 8 KB
constexpr uint32_t G_OFF_BAR = G_OFF_B + 128 * 32 * 2;
constexpr uint32_t G_OFF_TMEM = G_OFF_BAR + 8;
constexpr uint32_t G_SMEM = 56 * 1024;           // residency cap, not the footprint
constexpr uint32_t G_TMEM_COLS = 128;

// row r (of R) of an operand tile, K values k0 .. k0+31 (those >= ke read as 0):
// element (r, k) at P[r*ld + k] when kcontig, else at P[k*ld + r]; vec: P and
// ld allow 16-byte loads along K (k0 is a multiple of 32)
__device__ __forceinline__ void g_load(float (&v)[32], const float *__restrict__ P, int ld, bool kcontig, bool vec,
                                       int r, int R, int k0, int ke)
{
    if (r >= R) {
#pragma unroll
        for (int j = 0; j < 32; j++) v[j] = 0.f;
        return;
    }
    if (kcontig) {
        const float *row = P + (size_t)r * ld + k0;
#pragma unroll
        for (int q = 0; q < 8; q++) {
            if (vec && k0 + 4 * q + 4 <= ke) {
                const float4 t = __ldg(reinterpret_cast<const float4 *>(row + 4 * q));
                v[4 * q] = t.x; v[4 * q + 1] = t.y; v[4 * q + 2] = t.z; v[4 * q + 3] = t.w;
            } else {
#pragma unroll
                for (int j = 0; j < 4; j++) v[4 * q + j] = (k0 + 4 * q + j < ke) ? __ldg(row + 4 * q + j) : 0.f;
            }
        }
    } else {
#pragma unroll
        for (int j = 0; j < 32; j++) v[j] = (k0 + j < ke) ? __ldg(P + (size_t)(k0 + j) * ld + r) : 0.f;
    }
}

// row r of a 128 x 32 BF16 tile in the canonical layout: cano(r, 8o, 128) = o*2048 + r*16
__device__ __forceinline__ void g_store(unsigned char *tile, const float (&v)[32], uint32_t r)
{
#pragma unroll
    for (int o = 0; o < 4; o++) {
        uint4 w;
        w.x = pk_bf16(v[8 * o + 0], v[8 * o + 1]);
        w.y = pk_bf16(v[8 * o + 2], v[8 * o + 3]);
        w.z = pk_bf16(v[8 * o + 4], v[8 * o + 5]);
        w.w = pk_bf16(v[8 * o + 6], v[8 * o + 7]);
        *reinterpret_cast<uint4 *>(tile + cano(r, 8 * o, 128)) = w;
    }
}
}  // namespace

__global__ void __launch_bounds__(128) k_gemm_tc(int M, int N, int K, const float *__restrict__ A, int lda, int transA,
                                                 const float *__restrict__ B, int ldb, int transB, float *__restrict__ C,
                                                 int ldc, int kchunk, float *__restrict__ colsum, int *err)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    const uint32_t tid = threadIdx.x, warp = tid >> 5;
    const uint32_t sbase = smem_u32(smem);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + G_OFF_BAR);
    const int m0 = blockIdx.y * 128, n0 = blockIdx.x * 128;
    const int kb = blockIdx.z * kchunk, ke = min(K, kb + kchunk);
    C += (size_t)blockIdx.z * M * ldc;
    if (tid == 0) mbar_init(bar, 1);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sbase + G_OFF_TMEM),
                     "r"(G_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(smem + G_OFF_TMEM);
    const uint32_t lane_t = tmem + ((warp * 32u) << 16);
    constexpr uint32_t ID = idesc_bf16(128, 128);
    const bool kcA = !transA, kcB = transB != 0;
    const bool vecA = kcA && (lda & 3) == 0 && (reinterpret_cast<uintptr_t>(A) & 15) == 0;
    const bool vecB = kcB && (ldb & 3) == 0 && (reinterpret_cast<uintptr_t>(B) & 15) == 0;
    uint32_t phase = 0;
    bool ok = true, first = true;
    float a[32], b[32], bsum = 0.f;
    if (kb < ke) {
        g_load(a, A, lda, kcA, vecA, m0 + (int)tid, M, kb, ke);
        g_load(b, B, ldb, kcB, vecB, n0 + (int)tid, N, kb, ke);
    }
    for (int k0 = kb; k0 < ke; k0 += 32) {
        if (!first) {                          // the MMAs of the previous chunk have read the tiles
            ok = wait_all(bar, phase);
            phase ^= 1u;
            tc_fence_after();
            if (!ok) break;
        }
        g_store(smem + G_OFF_A, a, tid);
        g_store(smem + G_OFF_B, b, tid);
        if (colsum) {
#pragma unroll
            for (int j = 0; j < 32; j++) bsum += b[j];
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (uint32_t kk = 0; kk < 2; kk++)
                tc_mma(tmem, sdesc(sbase + G_OFF_A + kk * 2 * 2048, 2048, 128),
                       sdesc(sbase + G_OFF_B + kk * 2 * 2048, 2048, 128), ID, (first && kk == 0) ? 0u : 1u);
            tc_commit(sbase + G_OFF_BAR);
        }
        first = false;
        if (k0 + 32 < ke) {
            g_load(a, A, lda, kcA, vecA, m0 + (int)tid, M, k0 + 32, ke);
            g_load(b, B, ldb, kcB, vecB, n0 + (int)tid, N, k0 + 32, ke);
        }
    }
    if (ok && !first) {
        ok = wait_all(bar, phase);
        tc_fence_after();
    }
    if (ok) {
        const int row = m0 + (int)tid;
        const bool vecC = (ldc & 3) == 0 && (reinterpret_cast<uintptr_t>(C) & 15) == 0;
#pragma unroll 1
        for (uint32_t c = 0; c < 4 && n0 + 32 * (int)c < N; c++) {
            float v[32];
            if (first) {
#pragma unroll
                for (int j = 0; j < 32; j++) v[j] = 0.f;          // empty K range
            } else {
                tc_ld32(lane_t + 32 * c, v);
            }
            if (row >= M) continue;
            float *crow = C + (size_t)row * ldc;
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int col = n0 + 32 * (int)c + 4 * q;
                if (vecC && col + 4 <= N) {
                    *reinterpret_cast<float4 *>(crow + col) =
                        make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                } else {
#pragma unroll
                    for (int j = 0; j < 4; j++)
                        if (col + j < N) crow[col + j] = v[4 * q + j];
                }
            }
        }
    }
    if (ok && colsum && blockIdx.y == 0 && n0 + (int)tid < N) colsum[(size_t)blockIdx.z * N + n0 + tid] = bsum;
    if (!ok && tid == 0) atomicExch(err, 3);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(G_TMEM_COLS)
                     : "memory");
}

void launch_gemm_tc(ipfem_ctx *c, int M, int N, int K, const float *A, int lda, int transA, const float *B, int ldb,
                    int transB, float *C, int ldc, int kchunk, int splits, float *colsum)
{
    dim3 grid((N + 127) / 128, (M + 127) / 128, splits);
    k_gemm_tc<<<grid, 128, G_SMEM, c->stream>>>(M, N, K, A, lda, transA, B, ldb, transB, C, ldc, kchunk, colsum,
                                                c->d_err);
}

cudaError_t net_tc_configure()
{
    cudaError_t e = cudaFuncSetAttribute(k_patch_net_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_patch_net_bwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G_SMEM);
    return e;
}

void launch_patch_net_tc(ipfem_ctx *c, int64_t rows, const float *d_X, float *d_O, float *d_H1, float *d_H2)
{
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    const int64_t tiles = (rows + TC_ROWS - 1) / TC_ROWS;
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(tiles, 2 * (int64_t)sms));
    const MlpBuffers &m = c->mlp;
    k_patch_net_tc<<<grid, kNetThreads, TC_SMEM, c->stream>>>(
        rows, d_X, static_cast<const __nv_bfloat16 *>(m.w1t), static_cast<const __nv_bfloat16 *>(m.w2t),
        static_cast<const __nv_bfloat16 *>(m.w3t), m.params + kOffB1, m.params + kOffB2, m.params + kOffB3, d_O,
        d_H1, d_H2, c->d_err);
}

void launch_patch_net_bwd_tc(ipfem_ctx *c, int64_t rows, const float *d_dO, const float *d_H1, const float *d_H2,
                             float *d_dH2, float *d_dH1)
{
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    const int64_t tiles = (rows + TC_ROWS - 1) / TC_ROWS;
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(tiles, 2 * (int64_t)sms));
    k_patch_net_bwd_tc<<<grid, 128, TC_SMEM, c->stream>>>(rows, d_dO, d_H1, d_H2, c->mlp.params, d_dH2, d_dH1,
                                                          c->d_err);
}

}  // namespace ipfem
