// C-ABI of the learned preconditioner: initialisation, features, training
// (BF16 tensor-core forward/backward, Adam), and the flexible-CG solve with its
// fallback to Jacobi-PCG.  No counterpart in the reference.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>

#include "ipfem_internal.h"

using namespace ipfem;

namespace {

ipfem_status mfail(ipfem_ctx *c, ipfem_status s, const std::string &msg)
{
    if (c) c->err = msg;
    return s;
}

#define MK(expr)                                                                       \
    do {                                                                               \
        cudaError_t e_ = (expr);                                                       \
        if (e_ != cudaSuccess)                                                         \
            return mfail(c, e_ == cudaErrorMemoryAllocation ? IPFEM_OOM : IPFEM_CUDA,  \
                         std::string(#expr) + ": " + cudaGetErrorString(e_));          \
    } while (0)

template <class T>
cudaError_t alloc(T **p, size_t n)
{
    return cudaMalloc((void **)p, (n ? n : 1) * sizeof(T));
}

__global__ void k_gather_rows(int64_t rows, int width, const int64_t *__restrict__ idx, const float *__restrict__ src,
                              float *__restrict__ dst)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= rows * width) return;
    const int64_t r = i / width, c = i % width;
    dst[i] = src[idx[r] * width + c];
}

__global__ void k_to_float(int64_t n, const double *__restrict__ a, float *__restrict__ b)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

// T = e / (S * Dinv) per dof (0 where the dof is fixed)
__global__ void k_targets(int32_t n_nodes, const float *__restrict__ e, const float *__restrict__ S,
                          const float *__restrict__ dinv, float *__restrict__ T)
{
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_nodes) return;
    for (int k = 0; k < 2; k++) {
        const float d = dinv[2 * (int64_t)i + k];
        T[2 * (int64_t)i + k] = d > 0.f ? e[2 * (int64_t)i + k] / (S[i] * d) : 0.f;
    }
}

ipfem_status need_mlp(ipfem_ctx *c)
{
    if (!c) return IPFEM_INVALID;
    if (!c->mlp.ready) return mfail(c, IPFEM_INVALID, "ipfem_mlp_init not called");
    return IPFEM_OK;
}

}  // namespace

// FCG with the learned preconditioner on the FP32 tangent; falls back to the
// FP32 Jacobi-PCG (restarted from zero) when FCG stagnates or breaks down.
namespace ipfem {
ipfem_status fcg_device(ipfem_ctx *c, const double *d_b, double scale, double rtol, int max_it, int *iters,
                        int *fell_back)
{
    MixedBuffers &m = c->mx;
    *fell_back = 0;
    launch_fcg_init(c, d_b, scale, (float)rtol, max_it);
    c->launches += 3;
    const int batch = 16;
    if (!c->fcg_exec) {
        cudaGraph_t g = nullptr;
        MK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < batch; k++) launch_fcg_iteration(c);
        MK(cudaStreamEndCapture(c->stream, &g));
        cudaError_t e = cudaGraphInstantiate(&c->fcg_exec, g, 0);
        cudaGraphDestroy(g);
        MK(e);
    }
    int launched = 0;
    for (;;) {
        MK(cudaGraphLaunch(c->fcg_exec, c->stream));
        launched += batch;
        c->launches += 4 * batch;
        MK(cudaMemcpyAsync(m.h_sc, m.sc, sizeof(CGScalarsT<float>), cudaMemcpyDeviceToHost, c->stream));
        MK(cudaStreamSynchronize(c->stream));
        if (m.h_sc->done || launched >= max_it + batch) break;
    }
    MK(cudaGetLastError());
    int it = m.h_sc->iters;
    if (m.h_sc->done && m.h_sc->status == 0) {
        if (iters) *iters = it;
        return IPFEM_OK;
    }
    // stagnation, breakdown or iteration limit: Jacobi-PCG from zero
    *fell_back = 1;
    int it2 = 0;
    ipfem_status st = cg32_device(c, d_b, scale, rtol, max_it, &it2);
    if (iters) *iters = it + it2;
    return st;
}
}  // namespace ipfem

extern "C" {

ipfem_status ipfem_set_node_grid(ipfem_ctx *c, int32_t gr, int32_t gt)
{
    if (!c || gr < 1 || gt < 1 || (int64_t)gr * gt != c->s.n_nodes)
        return mfail(c, IPFEM_INVALID, "node grid does not match the number of nodes");
    c->mlp.gr = gr;
    c->mlp.gt = gt;
    return IPFEM_OK;
}

ipfem_status ipfem_mlp_init(ipfem_ctx *c, uint64_t seed)
{
    if (!c) return IPFEM_INVALID;
    if (c->precision != IPFEM_MIXED) return mfail(c, IPFEM_INVALID, "the learned preconditioner needs IPFEM_MIXED");
    MlpBuffers &m = c->mlp;
    const Setup &s = c->s;
    if (!m.params) {
        MK(alloc(&m.params, kMlpParams));
        MK(alloc(&m.grads, kMlpParams));
        MK(alloc(&m.m, kMlpParams));
        MK(alloc(&m.v, kMlpParams));
        MK(cudaMalloc(&m.w1t, 128 * 32 * 2));
        MK(cudaMalloc(&m.w2t, 128 * 128 * 2));
        MK(alloc(&m.pfrac, (size_t)s.n_nodes));
        MK(alloc(&m.pden, (size_t)s.n_nodes));
        MK(alloc(&m.r_old, (size_t)s.neq));
        MK(alloc(&m.loss, 1));
    }
    // He-uniform W1, W2; W3 = 0 and zero biases, so the initial network is Jacobi
    std::vector<float> p(kMlpParams, 0.f);
    std::mt19937_64 rng(seed);
    std::uniform_real_distribution<float> u(-1.f, 1.f);
    const float a1 = std::sqrt(6.f / 32.f), a2 = std::sqrt(6.f / 128.f);
    for (int i = 0; i < 32 * 128; i++) p[kOffW1 + i] = a1 * u(rng);
    for (int i = 0; i < 128 * 128; i++) p[kOffW2 + i] = a2 * u(rng);
    MK(cudaMemcpyAsync(m.params, p.data(), p.size() * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    MK(cudaMemsetAsync(m.m, 0, kMlpParams * sizeof(float), c->stream));
    MK(cudaMemsetAsync(m.v, 0, kMlpParams * sizeof(float), c->stream));
    MK(cudaMemsetAsync(m.grads, 0, kMlpParams * sizeof(float), c->stream));
    MK(cudaMemsetAsync(m.pfrac, 0, (size_t)s.n_nodes * sizeof(float), c->stream));
    m.adam_t = 0;
    MK(mlp_configure());
    mlp_pack_weights(c);
    MK(cudaStreamSynchronize(c->stream));
    MK(cudaGetLastError());
    m.ready = true;
    return IPFEM_OK;
}

ipfem_status ipfem_set_preconditioner(ipfem_ctx *c, int kind)
{
    if (!c || (kind != IPFEM_PREC_JACOBI && kind != IPFEM_PREC_MLP)) return mfail(c, IPFEM_INVALID, "bad preconditioner");
    if (kind == IPFEM_PREC_MLP) {
        if (c->precision != IPFEM_MIXED) return mfail(c, IPFEM_INVALID, "the learned preconditioner needs IPFEM_MIXED");
        if (!c->mlp.ready) return mfail(c, IPFEM_INVALID, "ipfem_mlp_init not called");
        if (c->mlp.gr == 0) return mfail(c, IPFEM_INVALID, "ipfem_set_node_grid not called");
    }
    c->preconditioner = kind;
    return IPFEM_OK;
}

ipfem_status ipfem_mlp_get_params(ipfem_ctx *c, float *out)
{
    ipfem_status st = need_mlp(c);
    if (st != IPFEM_OK) return st;
    MK(cudaMemcpyAsync(out, c->mlp.params, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    MK(cudaStreamSynchronize(c->stream));
    return IPFEM_OK;
}

ipfem_status ipfem_mlp_set_params(ipfem_ctx *c, const float *in)
{
    ipfem_status st = need_mlp(c);
    if (st != IPFEM_OK) return st;
    MK(cudaMemcpyAsync(c->mlp.params, in, kMlpParams * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    mlp_pack_weights(c);
    MK(cudaStreamSynchronize(c->stream));
    return IPFEM_OK;
}

ipfem_status ipfem_mlp_features(ipfem_ctx *c, const double *d_r, float *d_X, float *d_S)
{
    ipfem_status st = need_mlp(c);
    if (st != IPFEM_OK) return st;
    if (!d_r || !d_X || !d_S || c->mlp.gr == 0) return mfail(c, IPFEM_INVALID, "bad args or no node grid");
    const int64_t n = c->s.neq;
    k_to_float<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(n, d_r, c->mx.q);
    launch_plastic_fraction(c);
    launch_features(c, c->mx.q, d_X, d_S);
    c->launches += 5;
    MK(cudaStreamSynchronize(c->stream));
    MK(cudaGetLastError());
    return IPFEM_OK;
}

ipfem_status ipfem_mlp_targets(ipfem_ctx *c, const float *d_e, const float *d_S, float *d_T)
{
    ipfem_status st = need_mlp(c);
    if (st != IPFEM_OK) return st;
    if (!d_e || !d_S || !d_T) return mfail(c, IPFEM_INVALID, "bad args");
    k_targets<<<(c->s.n_nodes + 255) / 256, 256, 0, c->stream>>>(c->s.n_nodes, d_e, d_S, c->mx.dinv, d_T);
    c->launches += 1;
    MK(cudaStreamSynchronize(c->stream));
    MK(cudaGetLastError());
    return IPFEM_OK;
}

ipfem_status ipfem_mlp_forward(ipfem_ctx *c, const float *d_X, int64_t rows, float *d_O)
{
    ipfem_status st = need_mlp(c);
    if (st != IPFEM_OK) return st;
    if (!d_X || !d_O || rows < 0 || rows > ((int64_t)1 << 31) * 64) return mfail(c, IPFEM_INVALID, "bad args");
    if (rows == 0) return IPFEM_OK;
    launch_mlp_infer_rows(c, rows, d_X, d_O);
    c->launches += 1;
    MK(cudaStreamSynchronize(c->stream));
    MK(cudaGetLastError());
    return IPFEM_OK;
}

ipfem_status ipfem_mlp_grad(ipfem_ctx *c, const float *d_X, const float *d_Y, int64_t rows, float *grads, float *loss)
{
    ipfem_status st = need_mlp(c);
    if (st != IPFEM_OK) return st;
    if (!d_X || !d_Y || rows < 1 || rows > 65535LL * 64) return mfail(c, IPFEM_INVALID, "bad args (rows <= 4194240)");
    float *H1, *H2, *O, *dO, *dH1, *dH2;
    MK(alloc(&H1, (size_t)rows * 128));
    MK(alloc(&H2, (size_t)rows * 128));
    MK(alloc(&O, (size_t)rows * 2));
    MK(alloc(&dO, (size_t)rows * 2));
    MK(alloc(&dH1, (size_t)rows * 128));
    MK(alloc(&dH2, (size_t)rows * 128));
    mlp_train_step(c, rows, d_X, d_Y, H1, H2, O, dO, dH1, dH2, false, 0.f);
    c->launches += 16;
    if (grads) MK(cudaMemcpyAsync(grads, c->mlp.grads, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    if (loss) MK(cudaMemcpyAsync(loss, c->mlp.loss, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    MK(cudaStreamSynchronize(c->stream));
    cudaFree(H1); cudaFree(H2); cudaFree(O); cudaFree(dO); cudaFree(dH1); cudaFree(dH2);
    MK(cudaGetLastError());
    return IPFEM_OK;
}

ipfem_status ipfem_mlp_train(ipfem_ctx *c, const float *d_X, const float *d_Y, int64_t rows, int epochs, int batch,
                             float lr, uint64_t seed, float *loss_per_epoch)
{
    ipfem_status st = need_mlp(c);
    if (st != IPFEM_OK) return st;
    if (!d_X || !d_Y || rows < 1 || epochs < 0 || batch < 1 || batch > 65535 * 64)
        return mfail(c, IPFEM_INVALID, "bad args");
    const int64_t B = std::min<int64_t>(batch, rows);
    float *Xb, *Yb, *H1, *H2, *O, *dO, *dH1, *dH2;
    int64_t *d_idx;
    MK(alloc(&Xb, (size_t)B * 32));
    MK(alloc(&Yb, (size_t)B * 2));
    MK(alloc(&H1, (size_t)B * 128));
    MK(alloc(&H2, (size_t)B * 128));
    MK(alloc(&O, (size_t)B * 2));
    MK(alloc(&dO, (size_t)B * 2));
    MK(alloc(&dH1, (size_t)B * 128));
    MK(alloc(&dH2, (size_t)B * 128));
    MK(alloc(&d_idx, (size_t)rows));
    std::vector<int64_t> perm((size_t)rows);
    for (int64_t i = 0; i < rows; i++) perm[i] = i;
    std::mt19937_64 rng(seed);
    for (int ep = 0; ep < epochs; ep++) {
        std::shuffle(perm.begin(), perm.end(), rng);
        MK(cudaMemcpyAsync(d_idx, perm.data(), perm.size() * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream));
        double ls = 0.0;
        int nb = 0;
        for (int64_t b0 = 0; b0 + B <= rows; b0 += B) {
            k_gather_rows<<<(unsigned)((B * 32 + 255) / 256), 256, 0, c->stream>>>(B, 32, d_idx + b0, d_X, Xb);
            k_gather_rows<<<(unsigned)((B * 2 + 255) / 256), 256, 0, c->stream>>>(B, 2, d_idx + b0, d_Y, Yb);
            mlp_train_step(c, B, Xb, Yb, H1, H2, O, dO, dH1, dH2, true, lr);
            c->launches += 20;
            float l = 0.f;
            MK(cudaMemcpyAsync(&l, c->mlp.loss, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
            MK(cudaStreamSynchronize(c->stream));
            ls += l;
            nb++;
        }
        if (loss_per_epoch) loss_per_epoch[ep] = nb ? (float)(ls / nb) : 0.f;
    }
    MK(cudaStreamSynchronize(c->stream));
    cudaFree(Xb); cudaFree(Yb); cudaFree(H1); cudaFree(H2); cudaFree(O); cudaFree(dO); cudaFree(dH1); cudaFree(dH2);
    cudaFree(d_idx);
    MK(cudaGetLastError());
    return IPFEM_OK;
}

// FP32 Jacobi-CG on the current FP32 tangent with snapshots of (x_k, r_k) at
// iterations snap_iters[] (multiples of 32; k = 0 gives x_0 = 0, r_0 = b*scale)
// plus the final iterate; the right-hand side is scaled to unit norm.
ipfem_status ipfem_cg_snapshots(ipfem_ctx *c, const double *d_b, double rtol, int max_it, int n_snap,
                                const int32_t *snap_iters, float *d_xs, float *d_rs, float *d_xfinal, int *iters)
{
    if (!c || !d_b || n_snap < 0 || (n_snap && (!snap_iters || !d_xs || !d_rs)) || !d_xfinal)
        return mfail(c, IPFEM_INVALID, "bad args");
    if (c->precision != IPFEM_MIXED || !c->tangent_valid) return mfail(c, IPFEM_INVALID, "needs a mixed tangent");
    for (int k = 0; k < n_snap; k++)
        if (snap_iters[k] < 0 || snap_iters[k] % 32) return mfail(c, IPFEM_INVALID, "snapshot iterations: multiples of 32");
    MixedBuffers &m = c->mx;
    const size_t nb = (size_t)c->s.neq * sizeof(float);
    double bb = 0.0;
    {
        // |b| with the library's dot
        ipfem_status st = dot_host(c, d_b, d_b, &bb);
        if (st != IPFEM_OK) return st;
    }
    const double scale = bb > 0 ? 1.0 / std::sqrt(bb) : 1.0;
    launch_cg32_init(c, d_b, scale, (float)rtol, max_it);
    int done_it = 0;
    auto snap = [&](int it) -> ipfem_status {
        for (int k = 0; k < n_snap; k++)
            if (snap_iters[k] == it) {
                MK(cudaMemcpyAsync(d_xs + (size_t)k * c->s.neq, m.x, nb, cudaMemcpyDeviceToDevice, c->stream));
                MK(cudaMemcpyAsync(d_rs + (size_t)k * c->s.neq, m.r, nb, cudaMemcpyDeviceToDevice, c->stream));
            }
        return IPFEM_OK;
    };
    ipfem_status st = snap(0);
    if (st != IPFEM_OK) return st;
    for (;;) {
        for (int k = 0; k < 32; k++) launch_cg32_iteration(c);
        c->launches += 96;
        MK(cudaMemcpyAsync(m.h_sc, m.sc, sizeof(CGScalarsT<float>), cudaMemcpyDeviceToHost, c->stream));
        MK(cudaStreamSynchronize(c->stream));
        done_it += 32;
        if (m.h_sc->done || done_it >= max_it) break;
        st = snap(done_it);
        if (st != IPFEM_OK) return st;
    }
    MK(cudaMemcpyAsync(d_xfinal, m.x, nb, cudaMemcpyDeviceToDevice, c->stream));
    MK(cudaStreamSynchronize(c->stream));
    if (iters) *iters = m.h_sc->iters;
    MK(cudaGetLastError());
    return IPFEM_OK;
}

}  // extern "C"
