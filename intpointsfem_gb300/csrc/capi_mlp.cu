// C-ABI of the learned preconditioner: initialisation, features, the network
// forward, the training gradient pass and Adam (BF16 tensor-core GEMMs), and
// the flexible-CG solve with its fallback to Jacobi-PCG.  No counterpart in
// the reference.
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

ipfem_status need_mlp(ipfem_ctx *c)
{
    if (!c) return IPFEM_INVALID;
    if (!c->mlp.ready) return mfail(c, IPFEM_INVALID, "ipfem_mlp_init not called");
    return IPFEM_OK;
}

ipfem_status need_tangent(ipfem_ctx *c)
{
    ipfem_status st = need_mlp(c);
    if (st != IPFEM_OK) return st;
    if (c->precision != IPFEM_MIXED || !c->tangent_valid)
        return mfail(c, IPFEM_INVALID, "needs an assembled FP32 (IPFEM_MIXED) tangent");
    return IPFEM_OK;
}

// SELL slot of block (row, col) or -1
int32_t block_slot(const Setup &s, const SellLayout &L, int32_t row, int32_t col)
{
    const int32_t *c0 = s.col.data() + s.row_ptr[row], *c1 = s.col.data() + s.row_ptr[row + 1];
    const int32_t *f = std::lower_bound(c0, c1, col);
    return (f != c1 && *f == col) ? (int32_t)L.bsr_to_sell[s.row_ptr[row] + (f - c0)] : -1;
}

int32_t grid_nbr(int64_t i, int k, int32_t gr, int32_t gt)
{
    const int a = (int)(i % gr) + k % 3 - 1, b = (int)(i / gr) + k / 3 - 1;
    return (a < 0 || b < 0 || a >= gr || b >= gt) ? -1 : b * gr + a;
}

// slot[k][i]: FP32-tangent slot of block (i, nbr(i, k)) or -1
std::vector<int32_t> patch_slots(const Setup &s, const SellLayout &L, int32_t gr, int32_t gt)
{
    const int64_t n = s.n_nodes;
    std::vector<int32_t> slot((size_t)9 * n, -1);
    for (int64_t i = 0; i < n; i++)
        for (int k = 0; k < 9; k++) {
            const int32_t j = grid_nbr(i, k, gr, gt);
            if (j >= 0) slot[(size_t)k * n + i] = block_slot(s, L, (int32_t)i, j);
        }
    return slot;
}

// pslot[5k + l][i]: slot of block (nbr(i, k), nbr(i, l)) for k, l < 5, or -1
std::vector<int32_t> pair_slots(const Setup &s, const SellLayout &L, int32_t gr, int32_t gt)
{
    const int64_t n = s.n_nodes;
    std::vector<int32_t> slot((size_t)25 * n, -1);
    for (int64_t i = 0; i < n; i++)
        for (int k = 0; k < 5; k++) {
            const int32_t jk = grid_nbr(i, k, gr, gt);
            if (jk < 0) continue;
            for (int l = 0; l < 5; l++) {
                const int32_t jl = grid_nbr(i, l, gr, gt);
                if (jl >= 0) slot[(size_t)(5 * k + l) * n + i] = block_slot(s, L, jk, jl);
            }
        }
    return slot;
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
    if (!c->mlp.op_valid) launch_patch_operator(c);
    launch_fcg_init(c, d_b, scale, (float)rtol, max_it);
    c->launches += 3;
    const int batch = 16;
    if (!c->fcg_exec) {
        cudaGraph_t g = nullptr;
        MK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < batch; k++) launch_fcg_iteration(c, k & 1);
        MK(cudaStreamEndCapture(c->stream, &g));
        cudaError_t e = cudaGraphInstantiate(&c->fcg_exec, g, 0);
        cudaGraphDestroy(g);
        MK(e);
    }
    int launched = 0;
    for (;;) {
        MK(cudaGraphLaunch(c->fcg_exec, c->stream));
        launched += batch;
        c->launches += 3 * batch;
        MK(cudaMemcpyAsync(m.h_sc, m.sc, sizeof(CGScalarsT<float>), cudaMemcpyDeviceToHost, c->stream));
        MK(cudaStreamSynchronize(c->stream));
        if (m.h_sc->done || launched >= max_it + batch) break;
    }
    MK(cudaGetLastError());
    {
        // a bounded device wait that gave up is an error, not a result
        const ipfem_status e = check_device(c);
        if (e != IPFEM_OK) return e;
    }
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
    if (c->s.order != 2)
        return mfail(c, IPFEM_INVALID, "the learned preconditioner needs a grid of order-2 elements");
    if (c->mlp.ready && (gr != c->mlp.gr || gt != c->mlp.gt))
        return mfail(c, IPFEM_INVALID, "node grid is fixed once ipfem_mlp_init has run");
    c->mlp.gr = gr;
    c->mlp.gt = gt;
    return IPFEM_OK;
}

ipfem_status ipfem_mlp_init(ipfem_ctx *c, uint64_t seed)
{
    if (!c) return IPFEM_INVALID;
    if (c->precision != IPFEM_MIXED) return mfail(c, IPFEM_INVALID, "the learned preconditioner needs IPFEM_MIXED");
    if (c->mlp.gr == 0) return mfail(c, IPFEM_INVALID, "ipfem_set_node_grid not called");
    MlpBuffers &m = c->mlp;
    const Setup &s = c->s;
    if (!m.params) {
        MK(alloc(&m.params, kMlpParams));
        MK(alloc(&m.grads, kMlpParams));
        MK(alloc(&m.m, kMlpParams));
        MK(alloc(&m.v, kMlpParams));
        MK(cudaMalloc(&m.w1t, 128 * 32 * 2));
        MK(cudaMalloc(&m.w2t, 128 * 128 * 2));
        MK(cudaMalloc(&m.w3t, 24 * 128 * 2));
        MK(alloc(&m.X, (size_t)s.n_nodes * 32));
        MK(alloc(&m.O, (size_t)s.n_nodes * 20));
        MK(alloc(&m.M, (size_t)s.n_nodes * 20));
        MK(alloc(&m.r_old, (size_t)s.neq));
        MK(alloc(&m.y, (size_t)s.neq));
        MK(alloc(&m.p2, (size_t)s.neq));
        MK(cudaMalloc(&m.Gh, (size_t)s.n_nodes * 5 * 8));
        MK(alloc(&m.loss, 1));
        MK(alloc(&m.scal, 2));
        const std::vector<int32_t> slot = patch_slots(s, c->mx.sell, m.gr, m.gt);
        MK(alloc(&m.slot, slot.size()));
        MK(cudaMemcpyAsync(m.slot, slot.data(), slot.size() * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
        const std::vector<int32_t> pslot = pair_slots(s, c->mx.sell, m.gr, m.gt);
        MK(alloc(&m.pslot, pslot.size()));
        MK(cudaMemcpyAsync(m.pslot, pslot.data(), pslot.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                           c->stream));
        if (c->mx.have_sym) {
            // block codes of the upper-only layout: a lower block is -2 - slot of its stored twin
            const std::vector<int32_t> ss = patch_slots(s, c->mx.sym, m.gr, m.gt);
            MK(alloc(&m.slot_s, ss.size()));
            MK(cudaMemcpyAsync(m.slot_s, ss.data(), ss.size() * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
            const std::vector<int32_t> ps = pair_slots(s, c->mx.sym, m.gr, m.gt);
            MK(alloc(&m.pslot_s, ps.size()));
            MK(cudaMemcpyAsync(m.pslot_s, ps.data(), ps.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                               c->stream));
        }
        MK(cudaStreamSynchronize(c->stream));
        int64_t nf = 0;
        for (uint8_t f : s.fixed) nf += f ? 0 : 1;
        m.nf = (float)std::max<int64_t>(1, nf);
    }
    // He-uniform W1, W2; W3 = 0 and zero biases, so the initial operator is Jacobi
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
    if (!c || (kind != IPFEM_PREC_JACOBI && kind != IPFEM_PREC_MLP && kind != IPFEM_PREC_BLOCK_JACOBI))
        return mfail(c, IPFEM_INVALID, "bad preconditioner");
    if (kind == IPFEM_PREC_MLP) {
        if (c->precision != IPFEM_MIXED) return mfail(c, IPFEM_INVALID, "the learned preconditioner needs IPFEM_MIXED");
        if (!c->mlp.ready) return mfail(c, IPFEM_INVALID, "ipfem_mlp_init not called");
    }
    if (kind == IPFEM_PREC_BLOCK_JACOBI && !c->d_binv) {
        if (cudaMalloc((void **)&c->d_binv, (size_t)c->s.n_nodes * 4 * sizeof(double)) != cudaSuccess)
            return mfail(c, IPFEM_OOM, "allocation of the block-Jacobi inverses failed");
    }
    if (kind != c->preconditioner) {
        // the captured CG iterations launch the kernels of the previous preconditioner
        if (c->cg_exec) {
            cudaGraphExecDestroy(c->cg_exec);
            c->cg_exec = nullptr;
        }
        if (c->mx.exec) {
            cudaGraphExecDestroy(c->mx.exec);
            c->mx.exec = nullptr;
        }
    }
    c->preconditioner = kind;
    if (kind == IPFEM_PREC_BLOCK_JACOBI && c->tangent_valid) {
        launch_jacobi(c);
        MK(cudaStreamSynchronize(c->stream));
    }
    return IPFEM_OK;
}

ipfem_status ipfem_mlp_get_params(ipfem_ctx *c, float *out)
{
    ipfem_status st = need_mlp(c);
    if (st != IPFEM_OK) return st;
    if (!out) return mfail(c, IPFEM_INVALID, "bad args");
    MK(cudaMemcpyAsync(out, c->mlp.params, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    MK(cudaStreamSynchronize(c->stream));
    return IPFEM_OK;
}

ipfem_status ipfem_mlp_set_params(ipfem_ctx *c, const float *in)
{
    ipfem_status st = need_mlp(c);
    if (st != IPFEM_OK) return st;
    if (!in) return mfail(c, IPFEM_INVALID, "bad args");
    for (int i = 0; i < kMlpParams; i++)
        if (!std::isfinite(in[i])) return mfail(c, IPFEM_INVALID, "parameters are not finite");
    MK(cudaMemcpyAsync(c->mlp.params, in, kMlpParams * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    mlp_pack_weights(c);
    MK(cudaStreamSynchronize(c->stream));
    return IPFEM_OK;
}

ipfem_status ipfem_mlp_features(ipfem_ctx *c, float *d_X)
{
    ipfem_status st = need_tangent(c);
    if (st != IPFEM_OK) return st;
    if (!d_X) return mfail(c, IPFEM_INVALID, "bad args");
    launch_patch_features(c, d_X);
    c->launches += 1;
    MK(cudaStreamSynchronize(c->stream));
    MK(cudaGetLastError());
    return IPFEM_OK;
}

ipfem_status ipfem_mlp_forward(ipfem_ctx *c, const float *d_X, int64_t rows, float *d_O)
{
    ipfem_status st = need_mlp(c);
    if (st != IPFEM_OK) return st;
    if (!d_X || !d_O || rows < 0) return mfail(c, IPFEM_INVALID, "bad args");
    if (rows == 0) return IPFEM_OK;
    launch_patch_net(c, rows, d_X, d_O);
    c->launches += 1;
    MK(cudaStreamSynchronize(c->stream));
    MK(cudaGetLastError());
    return IPFEM_OK;
}

ipfem_status ipfem_mlp_operator(ipfem_ctx *c, float *d_M)
{
    ipfem_status st = need_tangent(c);
    if (st != IPFEM_OK) return st;
    if (!d_M) return mfail(c, IPFEM_INVALID, "bad args");
    if (!c->mlp.op_valid) launch_patch_operator(c);
    MK(cudaMemcpyAsync(d_M, c->mlp.M, (size_t)c->s.n_nodes * 20 * sizeof(float), cudaMemcpyDeviceToDevice,
                       c->stream));
    MK(cudaStreamSynchronize(c->stream));
    MK(cudaGetLastError());
    return IPFEM_OK;
}

ipfem_status ipfem_learn_grad(ipfem_ctx *c, const float *d_r, const float *d_e, int n_pairs, float w_kaporin,
                              float w_pairs, float *grads, float *loss)
{
    ipfem_status st = need_tangent(c);
    if (st != IPFEM_OK) return st;
    if (n_pairs < 0 || (n_pairs > 0 && (!d_r || !d_e)) || !(w_kaporin >= 0.f) || !(w_pairs >= 0.f) ||
        !std::isfinite(w_kaporin) || !std::isfinite(w_pairs))
        return mfail(c, IPFEM_INVALID, "bad args");
    MlpBuffers &m = c->mlp;
    const Setup &s = c->s;
    if (!m.H1) {
        const size_t n = (size_t)s.n_nodes;
        MK(alloc(&m.H1, n * 128));
        MK(alloc(&m.H2, n * 128));
        MK(alloc(&m.dH1, n * 128));
        MK(alloc(&m.dH2, n * 128));
        MK(alloc(&m.dN, n * 20));
        MK(alloc(&m.vec, (size_t)s.neq * 7));
        MK(alloc(&m.part, std::max(patch_part_floats(s.n_nodes), (size_t)2 * ((s.neq + 255) / 256))));
    }
    patch_learn_grad(c, d_r, d_e, n_pairs, w_kaporin, w_pairs);
    if (grads) MK(cudaMemcpyAsync(grads, m.grads, kMlpParams * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    if (loss) MK(cudaMemcpyAsync(loss, m.loss, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    MK(cudaStreamSynchronize(c->stream));
    MK(cudaGetLastError());
    return IPFEM_OK;
}

ipfem_status ipfem_mlp_adam(ipfem_ctx *c, const float *grads, float lr)
{
    ipfem_status st = need_mlp(c);
    if (st != IPFEM_OK) return st;
    if (!(lr > 0.f) || !std::isfinite(lr)) return mfail(c, IPFEM_INVALID, "bad learning rate");
    if (grads) {
        for (int i = 0; i < kMlpParams; i++)
            if (!std::isfinite(grads[i])) return mfail(c, IPFEM_NAN, "gradient is not finite");
        MK(cudaMemcpyAsync(c->mlp.grads, grads, kMlpParams * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    }
    mlp_adam_step(c, lr);
    MK(cudaStreamSynchronize(c->stream));
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
