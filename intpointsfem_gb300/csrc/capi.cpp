// C-ABI of libipfem: context lifecycle, the TPZElastoPlasticIntPointsStructMatrix
// calls (Assemble(rhs), Assemble(K, rhs)), the CG solve, the Newton driver of
// main.cpp, and the kernel-level replacements of TPZCudaCalls.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>

#include <nvtx3/nvToolsExt.h>

#include "ipfem_internal.h"

using namespace ipfem;

// NVTX range around a phase of the path (assemble, solve, commit): visible
// in Nsight timelines, free when no tool is attached
struct Range {
    explicit Range(const char *name) { nvtxRangePushA(name); }
    ~Range() { nvtxRangePop(); }
    Range(const Range &) = delete;
    Range &operator=(const Range &) = delete;
};

namespace {

// message of the last failed ipfem_create on this thread (no context exists then)
thread_local std::string t_create_err;

ipfem_status fail(ipfem_ctx *c, ipfem_status s, const std::string &msg)
{
    if (c) c->err = msg;
    return s;
}

#define CK(expr)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (expr);                                                          \
        if (e_ != cudaSuccess)                                                            \
            return fail(c, e_ == cudaErrorMemoryAllocation ? IPFEM_OOM : IPFEM_CUDA,      \
                        std::string(#expr) + ": " + cudaGetErrorString(e_));              \
    } while (0)

template <class T>
cudaError_t dalloc(T **p, size_t n)
{
    *p = nullptr;
    return cudaMalloc((void **)p, (n ? n : 1) * sizeof(T));
}

template <class T>
cudaError_t upload(T **p, const std::vector<T> &v, cudaStream_t st)
{
    cudaError_t e = dalloc(p, v.size());
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st);
}

cudaError_t upload_sell(const SellLayout &L, bool sorted, SellDev &D, cudaStream_t t)
{
    cudaError_t e = cudaSuccess;
    auto ck = [&](cudaError_t x) {
        if (x != cudaSuccess && e == cudaSuccess) e = x;
    };
    ck(upload(&D.slice_base, L.slice_base, t));
    ck(upload(&D.diag_blk, L.diag_blk, t));
    ck(upload(&D.sell_col, L.sell_col, t));
    ck(upload(&D.rowlen, L.rowlen, t));
    ck(upload(&D.sell_node, L.sell_node, t));
    ck(upload(&D.el_blk, L.el_blk, t));
    if (L.n_pat > 0) {
        ck(upload(&D.pat_id, L.pat_id, t));
        ck(upload(&D.pat_off, L.pat_off, t));
        D.n_pat = L.n_pat;
    }
    if (L.sym) {
        ck(upload(&D.tpat_id, L.tpat_id, t));
        ck(upload(&D.tpat_len, L.tpat_len, t));
        ck(upload(reinterpret_cast<int32_t **>(&D.tpat), L.tpat, t));
    }
    D.n_sell = L.n_sell;
    D.sorted = sorted;
    D.sym = L.sym;
    return e;
}

void free_sell(SellDev &D)
{
    void *ptrs[] = {D.slice_base, D.diag_blk, D.sell_col, D.rowlen, D.sell_node, D.el_blk, D.pat_id, D.pat_off,
                    D.tpat_id, D.tpat_len, D.tpat};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    D = SellDev();
}

void free_all(ipfem_ctx *c)
{
    free_sell(c->dsell);
    free_sell(c->mx.dsell);
    free_sell(c->mx.dsym);
    void *ptrs[] = {c->d_dphi, c->d_weight, c->d_mat, c->d_f0, c->d_df, c->d_lin, c->d_dofs, c->d_color_els, c->d_inc,
                    c->d_fixed, c->d_K,
                    c->d_dinv, c->d_eps_p, c->d_sigma, c->d_alpha, c->d_mtype, c->d_u, c->d_rhs, c->d_strain,
                    c->d_sigma_w, c->d_dep, c->d_fe, c->d_x, c->d_r, c->d_z, c->d_p, c->d_q, c->d_b, c->d_part,
                    c->d_sc, c->d_counters, c->d_dotres, c->d_err, c->d_acc, c->d_binv, c->d_u_prev};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    {
        MixedBuffers &m = c->mx;
        void *mp[] = {m.dphi, m.K, m.Ks, m.dinv, m.binv, m.x, m.r, m.z, m.p, m.q, m.part, m.sc, m.strain32, m.sigw32,
                      m.fe32, m.dphiT};
        for (void *p : mp)
            if (p) cudaFree(p);
        if (m.h_sc) cudaFreeHost(m.h_sc);
        if (m.exec) cudaGraphExecDestroy(m.exec);
    }
    if (c->h_sc) cudaFreeHost(c->h_sc);
    if (c->h_pin) cudaFreeHost(c->h_pin);
    if (c->cg_exec) cudaGraphExecDestroy(c->cg_exec);
    if (c->fcg_exec) cudaGraphExecDestroy(c->fcg_exec);
    {
        MlpBuffers &l = c->mlp;
        void *lp[] = {l.params, l.grads, l.m, l.v, l.w1t, l.w2t, l.w3t, l.slot, l.pslot, l.slot_s, l.pslot_s, l.X, l.O, l.M, l.y, l.Gh, l.p2, l.r_old, l.loss,
                      l.scal, l.H1, l.H2, l.dH1, l.dH2, l.dN, l.part, l.vec};
        for (void *p : lp)
            if (p) cudaFree(p);
    }
    if (c->ev_ready) {
        cudaEventDestroy(c->ev[0]);
        cudaEventDestroy(c->ev[1]);
    }
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->iter_log) std::fclose(c->iter_log);
}

}  // namespace

namespace ipfem {

// launch-error and device-error-word check after a synchronisation point
ipfem_status check_device(ipfem_ctx *c)
{
    CK(cudaGetLastError());
    int err = 0;
    CK(cudaMemcpyAsync(&c->h_pin[7], c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    std::memcpy(&err, &c->h_pin[7], sizeof(int));
    if (err)
        return fail(c, IPFEM_CUDA, err == kErrBulkWait ? "device wait timed out (bulk copy did not complete)"
                                                      : "device wait timed out (tensor-core pipeline)");
    return IPFEM_OK;
}

ipfem_status sync_check(ipfem_ctx *c)
{
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
    return check_device(c);
}

// the load factor and the load vector f0 + lambda df of the residuals that follow
void set_load(ipfem_ctx *c, double lambda)
{
    c->load_factor = lambda;
    launch_load_vector(c);
    c->launches += 1;
}

// residual of the current load factor at d_u into d_out (device)
void residual_device(ipfem_ctx *c, const double *d_u, double *d_out, int update_mem)
{
    c->launches += 4;
    if (c->res32_active && !update_mem) {
        MixedBuffers &m = c->mx;
        launch_gather_strain32(c, d_u, m.strain32);
        launch_compute_sigma32(c, 0, m.strain32, m.sigw32, nullptr);
        launch_stress_residual32(c, m.sigw32, m.fe32);
        launch_color_reduce32(c, m.fe32, 1, d_out);
        return;
    }
    launch_gather_strain(c, d_u, c->d_strain);
    launch_compute_sigma(c, update_mem, c->d_strain, c->d_sigma_w, nullptr);
    launch_stress_residual(c, c->d_sigma_w, c->d_fe);
    launch_color_reduce(c, c->d_fe, 1, d_out);
}

void tangent_device(ipfem_ctx *c, const double *d_u, double *d_out, int update_mem)
{
    c->launches += 6 + c->s.n_colors;
    if (c->res32_active && !update_mem) {
        MixedBuffers &m = c->mx;
        launch_gather_strain32(c, d_u, m.strain32);
        launch_compute_sigma32(c, 0, m.strain32, m.sigw32, c->d_dep);
        launch_stress_residual32(c, m.sigw32, m.fe32);
        launch_color_reduce32(c, m.fe32, 1, d_out);
    } else {
        launch_gather_strain(c, d_u, c->d_strain);
        launch_compute_sigma(c, update_mem, c->d_strain, c->d_sigma_w, c->d_dep);
        launch_stress_residual(c, c->d_sigma_w, c->d_fe);
        launch_color_reduce(c, c->d_fe, 1, d_out);
    }
    if (c->precision == 1) launch_stiffness32(c);
    else launch_stiffness(c);
    c->mlp.op_valid = false;     // the learned operator belongs to the previous tangent
    c->tangent_valid = true;
}

// CG on the current K with right-hand side d_b (device); solution in c->d_x
ipfem_status cg_device(ipfem_ctx *c, const double *d_b, double rtol, int max_it, int *iters)
{
    launch_cg_init(c, d_b, rtol, max_it);
    c->launches += 1;
    const int batch = 32;
    if (!c->cg_exec || c->cg_batch != batch) {
        if (c->cg_exec) {
            cudaGraphExecDestroy(c->cg_exec);
            c->cg_exec = nullptr;
        }
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < batch; k++) launch_cg_iteration(c);
        CK(cudaStreamEndCapture(c->stream, &g));
        cudaError_t e = cudaGraphInstantiate(&c->cg_exec, g, 0);
        cudaGraphDestroy(g);
        CK(e);
        c->cg_batch = batch;
    }
    int launched = 0;
    for (;;) {
        CK(cudaGraphLaunch(c->cg_exec, c->stream));
        launched += batch;
        c->launches += 3 * batch;
        CK(cudaMemcpyAsync(c->h_sc, c->d_sc, sizeof(CGScalars), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        if (c->h_sc->done || launched >= max_it + batch) break;
    }
    if (iters) *iters = c->h_sc->iters;
    ipfem_status st = check_device(c);
    if (st != IPFEM_OK) return st;
    if (!c->h_sc->done) return fail(c, IPFEM_NONCONVERGED, "CG did not finish");
    if (c->h_sc->status == IPFEM_BREAKDOWN) return fail(c, IPFEM_BREAKDOWN, "CG breakdown: p.Kp <= 0");
    if (c->h_sc->status == IPFEM_NONCONVERGED) return fail(c, IPFEM_NONCONVERGED, "CG reached max_it");
    if (!std::isfinite(c->h_sc->rr)) return fail(c, IPFEM_NAN, "CG residual is not finite");
    return IPFEM_OK;
}

// FP32 CG on the FP32 tangent for the right-hand side d_b * scale (d_b FP64,
// scale = 1/|b| so the FP32 system is well scaled); solution in c->mx.x
ipfem_status cg32_device(ipfem_ctx *c, const double *d_b, double scale, double rtol, int max_it, int *iters)
{
    MixedBuffers &m = c->mx;
    launch_cg32_init(c, d_b, scale, (float)rtol, max_it);
    c->launches += 1;
    const int batch = 32;
    if (!m.exec) {
        cudaGraph_t g = nullptr;
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < batch; k++) launch_cg32_iteration(c);
        CK(cudaStreamEndCapture(c->stream, &g));
        cudaError_t e = cudaGraphInstantiate(&m.exec, g, 0);
        cudaGraphDestroy(g);
        CK(e);
    }
    int launched = 0;
    for (;;) {
        CK(cudaGraphLaunch(m.exec, c->stream));
        launched += batch;
        c->launches += 3 * batch;
        CK(cudaMemcpyAsync(m.h_sc, m.sc, sizeof(CGScalarsT<float>), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        if (m.h_sc->done || launched >= max_it + batch) break;
    }
    if (iters) *iters = m.h_sc->iters;
    ipfem_status st = check_device(c);
    if (st != IPFEM_OK) return st;
    if (!m.h_sc->done) return fail(c, IPFEM_NONCONVERGED, "CG did not finish");
    if (m.h_sc->status == IPFEM_BREAKDOWN) return fail(c, IPFEM_BREAKDOWN, "CG breakdown: p.Kp <= 0");
    if (m.h_sc->status == IPFEM_NONCONVERGED) return fail(c, IPFEM_NONCONVERGED, "CG reached max_it");
    if (!std::isfinite(m.h_sc->rr)) return fail(c, IPFEM_NAN, "CG residual is not finite");
    return IPFEM_OK;
}

// K du = b in the context's precision; du accumulated into d_u (d_u += du)
// when add != 0, else written to c->d_x.
ipfem_status solve_device(ipfem_ctx *c, const double *d_b, double rtol, int max_it, int *iters, double *d_u, int add)
{
    if (c->precision == 0) {
        ipfem_status st = cg_device(c, d_b, rtol, max_it, iters);
        if (add) {
            launch_axpy_u(c, d_u, c->d_x);
            c->launches += 1;
        }
        return st;
    }
    double bb = 0.0;
    ipfem_status st = dot_host(c, d_b, d_b, &bb);
    if (st != IPFEM_OK) return st;
    const double bn = std::sqrt(bb);
    if (!(bn > 0.0)) {
        if (iters) *iters = 0;
        if (!add) CK(cudaMemsetAsync(c->d_x, 0, (size_t)c->s.neq * sizeof(double), c->stream));
        return std::isfinite(bn) ? IPFEM_OK : fail(c, IPFEM_NAN, "right-hand side is not finite");
    }
    if (c->preconditioner == IPFEM_PREC_MLP) {
        int fb = 0;
        st = fcg_device(c, d_b, 1.0 / bn, rtol, max_it, iters, &fb);
        c->fcg_fallbacks += fb;
    } else {
        st = cg32_device(c, d_b, 1.0 / bn, rtol, max_it, iters);
    }
    if (!add) {
        CK(cudaMemsetAsync(c->d_x, 0, (size_t)c->s.neq * sizeof(double), c->stream));
        launch_add_scaled32(c, c->d_x, c->mx.x, bn);
    } else {
        launch_add_scaled32(c, d_u, c->mx.x, bn);
    }
    c->launches += 1;
    return st;
}

// |v|^2 (canonical order) of a device vector, to the host
ipfem_status dot_host(ipfem_ctx *c, const double *a, const double *b, double *out)
{
    launch_dot(c, a, b, c->d_dotres);
    c->launches += 1;
    CK(cudaMemcpyAsync(&c->h_pin[0], c->d_dotres, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    *out = c->h_pin[0];
    return IPFEM_OK;
}

}  // namespace ipfem

void ipfem::set_thread_error(const std::string &msg)
{
    t_create_err = msg;
}

extern "C" {

const char *ipfem_status_string(ipfem_status s)
{
    switch (s) {
    case IPFEM_OK: return "ok";
    case IPFEM_NONCONVERGED: return "not converged";
    case IPFEM_NAN: return "non-finite value";
    case IPFEM_BREAKDOWN: return "CG breakdown";
    case IPFEM_OOM: return "out of device memory";
    case IPFEM_INVALID: return "invalid argument";
    case IPFEM_CUDA: return "CUDA error";
    case IPFEM_NO_DEVICE: return "no sm_103 device";
    }
    return "unknown";
}

const char *ipfem_last_error(const ipfem_ctx *c)
{
    return c ? c->err.c_str() : t_create_err.c_str();
}

void *ipfem_stream(ipfem_ctx *c)
{
    return c ? (void *)c->stream : nullptr;
}

ipfem_status ipfem_create(const ipfem_mesh *mesh, const ipfem_material *mat, ipfem_ctx **out)
{
    if (!out) return IPFEM_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        t_create_err = "no CUDA device";
        return IPFEM_NO_DEVICE;
    }
    ipfem_ctx *c = new (std::nothrow) ipfem_ctx();
    if (!c) return IPFEM_OOM;
    ipfem_status st = IPFEM_OK;
    auto bail = [&](ipfem_status s) {
        t_create_err = c->err.empty() ? ipfem_status_string(s) : c->err;
        free_all(c);
        delete c;
        return s;
    };
    t_create_err.clear();
    cudaGetDevice(&c->device);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, c->device) != cudaSuccess || prop.major != 10 || prop.minor != 3) {
        c->err = "libipfem is built for sm_103 (GB300) only";
        return bail(IPFEM_NO_DEVICE);
    }
    std::string msg = build_setup(mesh, mat, c->s);
    if (!msg.empty()) {
        c->err = msg;
        return bail(IPFEM_INVALID);
    }
    const Setup &s = c->s;
    auto ck = [&](cudaError_t e) {
        if (e != cudaSuccess && st == IPFEM_OK) st = (e == cudaErrorMemoryAllocation) ? IPFEM_OOM : IPFEM_CUDA;
    };
    ck(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    if (st != IPFEM_OK) return bail(st);
    cudaStream_t t = c->stream;
    ck(upload(&c->d_dphi, s.dphi, t));
    ck(upload(&c->d_weight, s.weight, t));
    ck(upload(&c->d_mat, s.mat, t));
    ck(upload(&c->d_f0, s.f0, t));
    ck(upload(&c->d_df, s.df, t));
    ck(dalloc(&c->d_lin, (size_t)s.neq));
    ck(upload(&c->d_dofs, s.dofs, t));
    ck(upload(&c->d_color_els, s.color_els, t));
    ck(upload(&c->d_inc, s.inc, t));
    ck(upload(&c->d_fixed, s.fixed, t));
    ck(upload_sell(s.sell, true, c->dsell, t));
    ck(dalloc(&c->d_K, (size_t)s.sell.n_sell * 4));
    ck(dalloc(&c->d_dinv, (size_t)s.neq));
    ck(dalloc(&c->d_eps_p, (size_t)s.n_ip * 4));
    ck(dalloc(&c->d_sigma, (size_t)s.n_ip * 4));
    ck(dalloc(&c->d_alpha, (size_t)s.n_ip));
    ck(dalloc(&c->d_mtype, (size_t)s.n_ip));
    ck(dalloc(&c->d_u, (size_t)s.neq));
    ck(dalloc(&c->d_rhs, (size_t)s.neq));
    ck(dalloc(&c->d_strain, (size_t)s.n_ip * 3));
    ck(dalloc(&c->d_sigma_w, (size_t)s.n_ip * 3));
    ck(dalloc(&c->d_dep, (size_t)s.n_ip * 9));
    ck(dalloc(&c->d_fe, (size_t)s.n_el * s.nd));
    ck(dalloc(&c->d_x, (size_t)s.neq));
    ck(dalloc(&c->d_r, (size_t)s.neq));
    ck(dalloc(&c->d_z, (size_t)s.neq));
    ck(dalloc(&c->d_p, (size_t)s.neq));
    ck(dalloc(&c->d_q, (size_t)s.neq));
    ck(dalloc(&c->d_b, (size_t)s.neq));
    c->n_red = (s.n_nodes + kRedBlock - 1) / kRedBlock;
    ck(dalloc(&c->d_part, (size_t)c->n_red * 3));
    ck(dalloc(&c->d_sc, 1));
    ck(dalloc(&c->d_counters, 16));
    ck(dalloc(&c->d_dotres, 8));
    ck(dalloc(&c->d_err, 1));
    ck(cudaMallocHost((void **)&c->h_sc, sizeof(CGScalars)));
    ck(cudaMallocHost((void **)&c->h_pin, 16 * sizeof(double)));
    if (st != IPFEM_OK) {
        c->err = "device allocation failed";
        return bail(st);
    }
    ck(cudaMemsetAsync(c->d_counters, 0, 16 * sizeof(unsigned), t));
    ck(cudaMemsetAsync(c->d_err, 0, sizeof(int), t));
    ck(cudaMemsetAsync(c->d_sc, 0, sizeof(CGScalars), t));
    ck(cudaMemsetAsync(c->d_u, 0, (size_t)s.neq * sizeof(double), t));
    ck(cudaMemsetAsync(c->d_K, 0, (size_t)s.sell.n_sell * 4 * sizeof(double), t));
    ck(cudaMemsetAsync(c->d_dinv, 0, (size_t)s.neq * sizeof(double), t));
    launch_load_vector(c);   // load factor 0
    ck(cudaGetLastError());
    // initial state: in-situ seed
    {
        std::vector<double> h((size_t)s.n_ip * 4);
        for (int k = 0; k < 4; k++) std::fill(h.begin() + k * s.n_ip, h.begin() + (k + 1) * s.n_ip, s.eps_p0[k]);
        ck(cudaMemcpyAsync(c->d_eps_p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, t));
        ck(cudaStreamSynchronize(t));
        for (int k = 0; k < 4; k++) std::fill(h.begin() + k * s.n_ip, h.begin() + (k + 1) * s.n_ip, s.sigma0[k]);
        ck(cudaMemcpyAsync(c->d_sigma, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, t));
        ck(cudaMemsetAsync(c->d_alpha, 0, (size_t)s.n_ip * sizeof(double), t));
        ck(cudaMemsetAsync(c->d_mtype, 0, (size_t)s.n_ip, t));
        ck(cudaStreamSynchronize(t));
    }
    if (st != IPFEM_OK) {
        c->err = "device initialisation failed";
        return bail(st);
    }
    *out = c;
    return IPFEM_OK;
}

void ipfem_destroy(ipfem_ctx *c)
{
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_all(c);
    delete c;
}

ipfem_status ipfem_sizes(const ipfem_ctx *c, int64_t out[6])
{
    if (!c || !out) return IPFEM_INVALID;
    out[0] = c->s.n_el;
    out[1] = c->s.n_ip;
    out[2] = c->s.n_nodes;
    out[3] = c->s.neq;
    out[4] = c->s.n_colors;
    out[5] = c->s.n_blocks;
    return IPFEM_OK;
}

ipfem_status ipfem_set_load_factor(ipfem_ctx *c, double lambda)
{
    if (!c) return IPFEM_INVALID;
    if (!std::isfinite(lambda)) return fail(c, IPFEM_INVALID, "load factor is not finite");
    set_load(c, lambda);
    CK(cudaGetLastError());
    return IPFEM_OK;
}

ipfem_status ipfem_set_precision(ipfem_ctx *c, int mode)
{
    if (!c || (mode != IPFEM_PLAIN_FP64 && mode != IPFEM_MIXED)) return fail(c, IPFEM_INVALID, "bad precision mode");
    if (mode == IPFEM_MIXED && !c->mx.dphi) {
        const Setup &s = c->s;
        MixedBuffers &m = c->mx;
        ipfem_status st = IPFEM_OK;
        auto ck = [&](cudaError_t e) {
            if (e != cudaSuccess && st == IPFEM_OK) st = (e == cudaErrorMemoryAllocation) ? IPFEM_OOM : IPFEM_CUDA;
        };
        std::vector<float> d32(s.dphi.begin(), s.dphi.end());
        d32.resize(d32.size() + 4, 0.f);   // the FP32 gather's last bulk copy may read 8 bytes past the blocks
        ck(upload(&m.dphi, d32, c->stream));
        const std::string e = build_sell(s, false, true, m.sell);
        if (!e.empty()) return fail(c, IPFEM_INVALID, e);
        build_row_stencils(m.sell);
        ck(upload_sell(m.sell, false, m.dsell, c->stream));
        // the upper-only layout where the grid has row and transposed stencils;
        // the values of the full layout are allocated when that layout is used
        m.have_sym = build_sell_sym(s, m.sym).empty();
        if (m.have_sym) {
            ck(upload_sell(m.sym, false, m.dsym, c->stream));
            ck(dalloc(&m.Ks, (size_t)m.sym.n_sell * 4));
        }
        if (!use_sym32(c)) ck(dalloc(&m.K, (size_t)m.sell.n_sell * 4));
        ck(dalloc(&m.dinv, (size_t)s.neq));
        ck(dalloc(&m.binv, (size_t)s.n_nodes * 4));
        ck(dalloc(&m.x, (size_t)s.neq));
        ck(dalloc(&m.r, (size_t)s.neq));
        ck(dalloc(&m.z, (size_t)s.neq));
        ck(dalloc(&m.p, (size_t)s.neq));
        ck(dalloc(&m.q, (size_t)s.neq));
        ck(dalloc(&m.part, (size_t)c->n_red * 2));
        ck(dalloc(&m.sc, 1));
        ck(cudaMallocHost((void **)&m.h_sc, sizeof(CGScalarsT<float>)));
        ck(cudaMemsetAsync(m.sc, 0, sizeof(CGScalarsT<float>), c->stream));
        ck(cudaStreamSynchronize(c->stream));
        if (st != IPFEM_OK) return fail(c, st, "allocation of the mixed-precision buffers failed");
    }
    if (mode != c->precision) c->tangent_valid = false;
    c->precision = mode;
    if (mode != IPFEM_MIXED) c->res32 = 0;
    return IPFEM_OK;
}

ipfem_status ipfem_set_update_mem(ipfem_ctx *c, int update)
{
    if (!c) return IPFEM_INVALID;
    c->update_mem = update ? 1 : 0;
    return IPFEM_OK;
}

static ipfem_status assemble_common(ipfem_ctx *c, const double *u, double *rhs, int where, bool tangent)
{
    if (!c || !u || !rhs || (where != IPFEM_HOST && where != IPFEM_DEVICE)) return fail(c, IPFEM_INVALID, "bad args");
    const size_t nb = (size_t)c->s.neq * sizeof(double);
    const double *du = u;
    double *dr = rhs;
    if (where == IPFEM_HOST) {
        CK(cudaMemcpyAsync(c->d_u, u, nb, cudaMemcpyHostToDevice, c->stream));
        du = c->d_u;
        dr = c->d_rhs;
    }
    // direct calls evaluate FP32 residuals whenever they are switched on (a
    // committing call stays FP64)
    c->res32_active = c->res32 && c->precision == IPFEM_MIXED;
    if (tangent) tangent_device(c, du, dr, c->update_mem);
    else residual_device(c, du, dr, c->update_mem);
    c->res32_active = 0;
    if (where == IPFEM_HOST) CK(cudaMemcpyAsync(rhs, dr, nb, cudaMemcpyDeviceToHost, c->stream));
    return sync_check(c);
}

ipfem_status ipfem_set_residual_precision(ipfem_ctx *c, int bits, double switch_rtol)
{
    if (!c) return IPFEM_INVALID;
    if (bits != 32 && bits != 64) return fail(c, IPFEM_INVALID, "residual precision must be 32 or 64 bits");
    if (!(switch_rtol >= 0.0 && switch_rtol < 1.0))
        return fail(c, IPFEM_INVALID, "switch_rtol must be in [0, 1)");
    if (bits == 32 && c->precision != IPFEM_MIXED)
        return fail(c, IPFEM_INVALID, "FP32 residuals need IPFEM_MIXED (its FP32 element blocks)");
    if (bits == 32 && !c->mx.strain32) {
        MixedBuffers &m = c->mx;
        const Setup &s = c->s;
        const size_t n_tiles = ((size_t)s.n_el + kTile32 - 1) / kTile32;
        cudaError_t e = dalloc(&m.strain32, (size_t)3 * s.n_ip);
        if (e == cudaSuccess) e = dalloc(&m.sigw32, (size_t)3 * s.n_ip);
        if (e == cudaSuccess) e = dalloc(&m.fe32, (size_t)s.n_el * s.nd);
        if (e == cudaSuccess) e = dalloc(&m.dphiT, n_tiles * kTile32 * 2 * (size_t)s.nn * (size_t)(s.nq | 1));
        if (e != cudaSuccess)
            return fail(c, e == cudaErrorMemoryAllocation ? IPFEM_OOM : IPFEM_CUDA,
                        "allocation of the FP32 residual buffers failed");
        launch_tile_blocks32(c);
        c->launches += 1;
        CK(cudaGetLastError());
    }
    c->res32 = bits == 32;
    c->res32_switch = switch_rtol;
    return IPFEM_OK;
}

ipfem_status ipfem_assemble_residual(ipfem_ctx *c, const double *u, double *rhs, int where)
{
    return assemble_common(c, u, rhs, where, false);
}

ipfem_status ipfem_set_newton_accel(ipfem_ctx *c, int mode)
{
    if (!c || (mode != 0 && mode != 1)) return fail(c, IPFEM_INVALID, "bad Newton acceleration mode");
    if (mode == 1 && c->inner.mode == 1)
        return fail(c, IPFEM_INVALID, "the modified-Thomas acceleration needs a fixed inner tolerance (its step "
                                      "factor assumes accurate inner solves)");
    if (mode == 1 && !c->d_acc) {
        cudaError_t e = dalloc(&c->d_acc, (size_t)c->s.neq);
        if (e != cudaSuccess) return fail(c, IPFEM_OOM, "allocation of the acceleration vector failed");
    }
    c->newton_accel = mode;
    return IPFEM_OK;
}

ipfem_status ipfem_set_newton_tangent(ipfem_ctx *c, int mode)
{
    if (!c || (mode != 0 && mode != 1)) return fail(c, IPFEM_INVALID, "bad Newton tangent mode");
    c->newton_tangent = mode;
    return IPFEM_OK;
}

ipfem_status ipfem_set_row_stencils(ipfem_ctx *c, int on)
{
    if (!c || (on != 0 && on != 1)) return fail(c, IPFEM_INVALID, "bad row-stencil mode");
    if (on != c->row_stencils) {
        // captured CG iterations launch the SpMV of the previous mode
        cudaGraphExec_t *g[] = {&c->cg_exec, &c->fcg_exec, &c->mx.exec};
        for (cudaGraphExec_t *e : g)
            if (*e) {
                cudaGraphExecDestroy(*e);
                *e = nullptr;
            }
    }
    // with the upper-only FP32 layout the switch also selects the layout the
    // FP32 tangent lives in: it has to be assembled again
    if (on != c->row_stencils && c->mx.have_sym) c->tangent_valid = false;
    if (!on && c->mx.have_sym && !c->mx.K) {
        const cudaError_t e = dalloc(&c->mx.K, (size_t)c->mx.sell.n_sell * 4);
        if (e != cudaSuccess)
            return fail(c, e == cudaErrorMemoryAllocation ? IPFEM_OOM : IPFEM_CUDA,
                        "allocation of the full-layout FP32 tangent failed");
    }
    c->row_stencils = on;
    return IPFEM_OK;
}

ipfem_status ipfem_row_stencil_count(ipfem_ctx *c, int32_t *n_fp64, int32_t *n_fp32)
{
    if (!c) return IPFEM_INVALID;
    if (n_fp64) *n_fp64 = c->dsell.n_pat;
    if (n_fp32) *n_fp32 = c->mx.dsell.n_pat;
    return IPFEM_OK;
}

ipfem_status ipfem_layout_info(ipfem_ctx *c, int fp32, int64_t *stored_blocks, int64_t *slots,
                               int32_t *upper_only)
{
    if (!c) return IPFEM_INVALID;
    if (fp32 && c->precision != IPFEM_MIXED)
        return fail(c, IPFEM_INVALID, "no FP32 tangent: the precision is not IPFEM_MIXED");
    const int64_t nb = c->s.n_blocks, nn = c->s.n_nodes;
    const bool sym = fp32 && use_sym32(c);
    // the block pattern is symmetric: n_blocks = n_nodes + 2 * (off-diagonal upper blocks)
    if (stored_blocks) *stored_blocks = sym ? (nb + nn) / 2 : nb;
    if (slots) *slots = !fp32 ? c->s.sell.n_sell : (sym ? c->mx.sym.n_sell : c->mx.sell.n_sell);
    if (upper_only) *upper_only = sym ? 1 : 0;
    return IPFEM_OK;
}

ipfem_status ipfem_assemble(ipfem_ctx *c, const double *u, double *rhs, int where)
{
    return assemble_common(c, u, rhs, where, true);
}

ipfem_status ipfem_get_stiffness(ipfem_ctx *c, int64_t *row_ptr, int32_t *col, double *vals)
{
    if (!c) return IPFEM_INVALID;
    const Setup &s = c->s;
    if (row_ptr) std::memcpy(row_ptr, s.row_ptr.data(), s.row_ptr.size() * sizeof(int64_t));
    if (col) std::memcpy(col, s.col.data(), s.col.size() * sizeof(int32_t));
    if (vals && c->precision == 1) {
        const bool sym = use_sym32(c);
        const SellLayout &L = sym ? c->mx.sym : c->mx.sell;
        std::vector<float> h((size_t)L.n_sell * 4);
        CK(cudaMemcpyAsync(h.data(), sym ? c->mx.Ks : c->mx.K, h.size() * sizeof(float), cudaMemcpyDeviceToHost,
                           c->stream));
        CK(cudaStreamSynchronize(c->stream));
        for (int64_t k = 0; k < s.n_blocks; k++) {
            const int64_t code = L.bsr_to_sell[k];
            if (code >= 0) {
                for (int j = 0; j < 4; j++) vals[4 * k + j] = h[4 * code + j];
            } else {
                // a lower block of the upper-only layout: the transpose of its stored twin
                const float *t = &h[4 * (-2 - code)];
                vals[4 * k + 0] = t[0];
                vals[4 * k + 1] = t[2];
                vals[4 * k + 2] = t[1];
                vals[4 * k + 3] = t[3];
            }
        }
    } else if (vals) {
        std::vector<double> h((size_t)s.sell.n_sell * 4);
        CK(cudaMemcpyAsync(h.data(), c->d_K, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        for (int64_t k = 0; k < s.n_blocks; k++)
            std::memcpy(vals + 4 * k, h.data() + 4 * s.sell.bsr_to_sell[k], 4 * sizeof(double));
    }
    return IPFEM_OK;
}

ipfem_status ipfem_get_stiffness_sym_csr(ipfem_ctx *c, int64_t *nnz, int64_t *ia, int64_t *ja, double *a)
{
    if (!c || !nnz) return fail(c, IPFEM_INVALID, "bad args");
    const Setup &s = c->s;
    // entries of the upper triangle: 4 per off-diagonal block (j > i) of a
    // block row, 3 per diagonal block ((2i, 2i), (2i, 2i+1), (2i+1, 2i+1))
    int64_t n_up = 0;
    for (int32_t i = 0; i < s.n_nodes; i++)
        for (int64_t k = s.row_ptr[i]; k < s.row_ptr[i + 1]; k++) n_up += s.col[k] > i ? 4 : (s.col[k] == i ? 3 : 0);
    if (!ia && !ja && !a) {
        *nnz = n_up;
        return IPFEM_OK;
    }
    if (*nnz < n_up) return fail(c, IPFEM_INVALID, "ipfem_get_stiffness_sym_csr: arrays hold fewer than nnz entries");
    if (!ia || !ja) return fail(c, IPFEM_INVALID, "ipfem_get_stiffness_sym_csr: ia and ja are needed");
    std::vector<double> v;
    if (a) {
        if (!c->tangent_valid) return fail(c, IPFEM_INVALID, "no tangent assembled");
        v.resize((size_t)s.n_blocks * 4);
        ipfem_status st = ipfem_get_stiffness(c, nullptr, nullptr, v.data());
        if (st != IPFEM_OK) return st;
    }
    // dof row 2i+p holds, for the blocks (i, j >= i) in ascending j, the
    // columns 2j and 2j+1 at or right of the diagonal: columns ascend
    int64_t e = 0;
    ia[0] = 0;
    for (int32_t i = 0; i < s.n_nodes; i++) {
        for (int p = 0; p < 2; p++) {
            const int64_t row = 2 * (int64_t)i + p;
            for (int64_t k = s.row_ptr[i]; k < s.row_ptr[i + 1]; k++) {
                const int32_t j = s.col[k];
                if (j < i) continue;
                for (int q = 0; q < 2; q++) {
                    const int64_t col = 2 * (int64_t)j + q;
                    if (col < row) continue;
                    ja[e] = col;
                    if (a) a[e] = v[4 * k + 2 * p + q];
                    e++;
                }
            }
            ia[row + 1] = e;
        }
    }
    *nnz = e;
    return IPFEM_OK;
}

ipfem_status ipfem_solve(ipfem_ctx *c, const double *b, double *x, double rtol, int max_it, int where, int *iters)
{
    if (!c || !b || !x || !(rtol >= 0) || (where != IPFEM_HOST && where != IPFEM_DEVICE))
        return fail(c, IPFEM_INVALID, "bad args");
    if (!c->tangent_valid) return fail(c, IPFEM_INVALID, "no tangent assembled");
    const size_t nb = (size_t)c->s.neq * sizeof(double);
    const double *db = b;
    if (where == IPFEM_HOST) {
        CK(cudaMemcpyAsync(c->d_b, b, nb, cudaMemcpyHostToDevice, c->stream));
        db = c->d_b;
    }
    ipfem_status st = solve_device(c, db, rtol, max_it, iters, nullptr, 0);
    if (where == IPFEM_HOST) CK(cudaMemcpyAsync(x, c->d_x, nb, cudaMemcpyDeviceToHost, c->stream));
    else if (x != c->d_x) CK(cudaMemcpyAsync(x, c->d_x, nb, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return st;
}

// Assemble(K, rhs) of a Newton iteration, or Assemble(rhs) alone in the
// initial-stiffness mode once a tangent exists (the reference's logged runs:
// the linear solve reuses the K of the first assembly, main.cpp:218-222 with
// AssembleResidual per iteration)
static void newton_assemble(ipfem_ctx *c, double *du)
{
    if (c->newton_tangent == 1 && c->ns.have_k) {
        residual_device(c, du, c->d_rhs, 0);
    } else {
        tangent_device(c, du, c->d_rhs, 0);
        c->ns.have_k = 1;
    }
}

// One Newton iteration of the load-stepped solve (main.cpp:185-256): CG on the
// current tangent, u += du, Assemble(K, rhs), convergence test; a load step
// that converges (or reaches newton_max_it) is accepted (state commit,
// main.cpp:487-522) and the next step's first assembly happens at the start
// of the following iteration.
static ipfem_status newton_advance(ipfem_ctx *c, int32_t n_iters, double *du, ipfem_solve_stats *st, double *log,
                                   int32_t log_cap, int32_t *nlog)
{
    NewtonState &ns = c->ns;
    const ipfem_solve_opts &o = ns.opts;
    cudaEvent_t *ev = c->ev;
    auto elapsed = [&]() {
        float ms = 0;
        cudaEventSynchronize(ev[1]);
        cudaEventElapsedTime(&ms, ev[0], ev[1]);
        return (double)ms;
    };
    int32_t done = 0;
    while (done < n_iters && ns.step < ns.step_end) {
        const double ma0 = st->ms_assemble, ms0 = st->ms_solve, mc0 = st->ms_commit;
        if (!ns.open) {
            Range rg("ipfem:newton:first_assembly");
            set_load(c, (double)(ns.step + 1) / (double)o.n_steps);
            c->res32_active = c->res32 && c->precision == IPFEM_MIXED;
            cudaEventRecord(ev[0], c->stream);
            double r0sq = -1.0;
            if (c->predictor) {
                // the step's convergence target is |R| at the last accepted
                // solution, as without the predictor; then the secant
                // predictor (equal load increments) moves u by the last step's
                // displacement increment before the first assembly
                if (ns.have_prev) {
                    residual_device(c, du, c->d_rhs, 0);
                    ipfem_status e = dot_host(c, c->d_rhs, c->d_rhs, &r0sq);
                    if (e != IPFEM_OK) return e;
                    launch_predict(c, du, c->d_u_prev, 1.0);
                } else {
                    CK(cudaMemcpyAsync(c->d_u_prev, du, (size_t)c->s.neq * sizeof(double), cudaMemcpyDeviceToDevice,
                                       c->stream));
                }
                c->launches += 1;
            }
            newton_assemble(c, du);
            cudaEventRecord(ev[1], c->stream);
            double rsq = 0;
            ipfem_status e = dot_host(c, c->d_rhs, c->d_rhs, &rsq);
            st->ms_assemble += elapsed();
            if (e != IPFEM_OK) return e;
            ns.r0 = std::sqrt(r0sq >= 0.0 ? r0sq : rsq);
            ns.rn = std::sqrt(rsq);
            ns.r_pred = ns.rn;
            ns.it = 0;
            ns.alpha = 1.0;
            ns.open = 1;
            if (!std::isfinite(ns.r0) || !std::isfinite(ns.rn)) return fail(c, IPFEM_NAN, "residual is not finite");
        }
        // a predicted start may already meet the step's target
        bool conv = (ns.r0 == 0.0) || (!c->res32_active && ns.rn <= o.newton_rtol * ns.r0);
        if (!conv) {
            // inner tolerance of this Newton iteration
            double eta = o.cg_rtol;
            if (c->inner.mode == 1 && ns.it > 0) {
                const InnerTolerance &t = c->inner;
                const double ratio = ns.rn / ns.rn_prev;
                if (ratio > 0.9) {
                    // stagnating or growing |R|: the forcing term would loosen
                    // the solve just when the Newton step needs to be accurate
                    eta = t.eta_min;
                } else {
                    eta = t.gamma * std::pow(ratio, t.alpha);
                    const double carry = t.gamma * std::pow(ns.eta, t.alpha);
                    if (carry > 0.1) eta = std::max(eta, carry);
                    eta = std::max(eta, 0.5 * o.newton_rtol * ns.r0 / ns.rn);
                    eta = std::min(std::max(eta, t.eta_min), t.eta_max);
                }
            }
            ns.eta = eta;
            int k = 0;
            const int64_t fb0 = c->fcg_fallbacks;
            Range rg("ipfem:newton:iteration");
            cudaEventRecord(ev[0], c->stream);
            ipfem_status e;
            {
                Range rs("ipfem:solve");
                e = solve_device(c, c->d_rhs, eta, o.cg_max_it, &k, du, c->newton_accel ? 0 : 1);
            }
            st->fcg_fallbacks += c->fcg_fallbacks - fb0;
            cudaEventRecord(ev[1], c->stream);
            st->ms_solve += elapsed();
            st->cg_iters += k;
            if (e != IPFEM_OK && e != IPFEM_NONCONVERGED) return e;
            if (c->newton_accel) {
                // modified-Thomas acceleration (main.cpp:194-217): u += alpha du,
                // residual at u, a second solve with the same tangent, alpha +=
                // (alpha du . du~) / (alpha du . alpha du), u += du~
                launch_scale_add(c, du, c->d_x, ns.alpha, c->d_acc);
                cudaEventRecord(ev[0], c->stream);
                residual_device(c, du, c->d_rhs, 0);
                cudaEventRecord(ev[1], c->stream);
                st->ms_assemble += elapsed();
                int k2 = 0;
                const int64_t fb1 = c->fcg_fallbacks;
                cudaEventRecord(ev[0], c->stream);
                e = solve_device(c, c->d_rhs, eta, o.cg_max_it, &k2, du, 0);
                st->fcg_fallbacks += c->fcg_fallbacks - fb1;
                cudaEventRecord(ev[1], c->stream);
                st->ms_solve += elapsed();
                st->cg_iters += k2;
                k += k2;
                if (e != IPFEM_OK && e != IPFEM_NONCONVERGED) return e;
                double num = 0.0, dem = 0.0;
                e = dot_host(c, c->d_acc, c->d_x, &num);
                if (e == IPFEM_OK) e = dot_host(c, c->d_acc, c->d_acc, &dem);
                if (e != IPFEM_OK) return e;
                if (dem > 0.0) ns.alpha = ns.alpha + num / dem;
                launch_axpy_u(c, du, c->d_x);
                c->launches += 2;
            }
            ns.it++;
            done++;
            st->newton_iters++;
            Range ra("ipfem:assemble");
            cudaEventRecord(ev[0], c->stream);
            newton_assemble(c, du);
            cudaEventRecord(ev[1], c->stream);
            double rsq = 0;
            e = dot_host(c, c->d_rhs, c->d_rhs, &rsq);
            st->ms_assemble += elapsed();
            if (e != IPFEM_OK) return e;
            const double rn_prev = ns.rn;
            ns.rn_prev = rn_prev;
            ns.rn = std::sqrt(rsq);
            if (!std::isfinite(ns.rn)) return fail(c, IPFEM_NAN, "residual is not finite");
            const int was32 = c->res32_active;
            const double rsq32 = rsq;
            if (c->res32_active && (ns.rn <= c->res32_switch * ns.r0 || ns.rn > 0.5 * rn_prev)) {
                // FP64 refinement: from here on this load step evaluates FP64
                // residuals, starting with the one at the current u (the
                // tangent just assembled is kept); the convergence test only
                // ever sees FP64 residuals
                c->res32_active = 0;
                cudaEventRecord(ev[0], c->stream);
                residual_device(c, du, c->d_rhs, 0);
                cudaEventRecord(ev[1], c->stream);
                e = dot_host(c, c->d_rhs, c->d_rhs, &rsq);
                st->ms_assemble += elapsed();
                if (e != IPFEM_OK) return e;
                ns.rn = std::sqrt(rsq);
                if (!std::isfinite(ns.rn)) return fail(c, IPFEM_NAN, "residual is not finite");
            }
            if (log && *nlog < log_cap) {
                log[3 * *nlog + 0] = (double)ns.step;
                log[3 * *nlog + 1] = (double)k;
                log[3 * *nlog + 2] = ns.rn;
                (*nlog)++;
            }
            conv = !c->res32_active && ns.rn <= o.newton_rtol * ns.r0;
            if (c->iter_log) {
                const double ma = st->ms_assemble - ma0, ms = st->ms_solve - ms0;
                std::fprintf(c->iter_log,
                             "{\"step\": %d, \"iter\": %d, \"cg_iters\": %d, \"res\": %.17g, \"res_rel\": %.17g, "
                             "\"ms_solve\": %.6f, \"ms_assemble\": %.6f, \"ips_assemble\": %.6g, "
                             "\"fcg_fallback\": %d, \"res32\": %d, \"res32_rel\": %.17g, \"cg_rtol\": %.6g}\n",
                             ns.step, ns.it, k, ns.rn, ns.r0 > 0.0 ? ns.rn / ns.r0 : 0.0, ms, ma,
                             ma > 0.0 ? (double)c->s.n_ip / (1e-3 * ma) : 0.0,
                             (int)(c->fcg_fallbacks - fb0), c->res32_active,
                             was32 && ns.r0 > 0.0 ? std::sqrt(rsq32) / ns.r0 : 0.0, eta);
                std::fflush(c->iter_log);
            }
        }
        if (conv || ns.it >= o.newton_max_it) {
            st->last_step_iters = ns.it;
            st->final_res = ns.r0 > 0.0 ? ns.rn / ns.r0 : 0.0;
            if (!conv) ns.all_converged = 0;
            {
                Range rc("ipfem:commit");
                cudaEventRecord(ev[0], c->stream);
                residual_device(c, du, c->d_b, 1);
                cudaEventRecord(ev[1], c->stream);
                st->ms_commit += elapsed();
            }
            ipfem_status e = sync_check(c);
            if (e != IPFEM_OK) return e;
            if (c->iter_log) {
                std::fprintf(c->iter_log,
                             "{\"step\": %d, \"accepted\": true, \"newton_iters\": %d, \"converged\": %s, "
                             "\"res_rel\": %.17g, \"res_start_rel\": %.17g, \"ms_commit\": %.6f, "
                             "\"ms_step_total\": %.6f}\n",
                             ns.step, ns.it, conv ? "true" : "false", ns.r0 > 0.0 ? ns.rn / ns.r0 : 0.0,
                             ns.r0 > 0.0 ? ns.r_pred / ns.r0 : 0.0,
                             st->ms_commit - mc0,
                             (st->ms_assemble - ma0) + (st->ms_solve - ms0) + (st->ms_commit - mc0));
                std::fflush(c->iter_log);
            }
            ns.step++;
            ns.open = 0;
            ns.have_prev = c->predictor;   // d_u_prev holds the start of the step just accepted
        }
    }
    st->converged = ns.all_converged;
    return IPFEM_OK;
}

ipfem_status ipfem_set_consistent_tangent(ipfem_ctx *c, int on)
{
    if (!c || (on != 0 && on != 1)) return fail(c, IPFEM_INVALID, "consistent tangent must be 0 or 1");
    c->consistent_tangent = on;
    c->tangent_valid = false;   // the next solve needs a tangent of the chosen kind
    return IPFEM_OK;
}

ipfem_status ipfem_set_spectral_mode(ipfem_ctx *c, int mode)
{
    if (!c || (mode != 0 && mode != 1)) return fail(c, IPFEM_INVALID, "spectral mode must be 0 or 1");
    c->spectral_mode = mode;
    c->tangent_valid = false;   // the tangent depends on the decomposition
    return IPFEM_OK;
}

ipfem_status ipfem_set_newton_predictor(ipfem_ctx *c, int on)
{
    if (!c || (on != 0 && on != 1)) return fail(c, IPFEM_INVALID, "predictor must be 0 or 1");
    if (on && !c->d_u_prev) {
        const cudaError_t e = dalloc(&c->d_u_prev, (size_t)c->s.neq);
        if (e != cudaSuccess) return fail(c, IPFEM_OOM, "allocation of the predictor vector failed");
    }
    c->predictor = on;
    c->ns.have_prev = 0;   // the next load step starts unpredicted
    return IPFEM_OK;
}

ipfem_status ipfem_set_inner_tolerance(ipfem_ctx *c, int mode, double gamma, double alpha, double eta_min,
                                       double eta_max)
{
    if (!c) return IPFEM_INVALID;
    if (mode != 0 && mode != 1) return fail(c, IPFEM_INVALID, "inner tolerance mode must be 0 or 1");
    if (mode == 1 && c->newton_accel)
        return fail(c, IPFEM_INVALID, "the adaptive inner tolerance cannot be combined with the modified-Thomas "
                                      "acceleration (its step factor assumes accurate inner solves)");
    if (mode == 1 && !(gamma > 0.0 && gamma <= 1.0 && alpha > 1.0 && alpha <= 2.0 && eta_min > 0.0 &&
                       eta_min <= eta_max && eta_max < 1.0))
        return fail(c, IPFEM_INVALID, "need 0 < gamma <= 1, 1 < alpha <= 2 and 0 < eta_min <= eta_max < 1");
    c->inner.mode = mode;
    if (mode == 1) {
        c->inner.gamma = gamma;
        c->inner.alpha = alpha;
        c->inner.eta_min = eta_min;
        c->inner.eta_max = eta_max;
    }
    return IPFEM_OK;
}

ipfem_status ipfem_newton_begin(ipfem_ctx *c, const ipfem_solve_opts *o, int32_t s0, int32_t s1)
{
    if (!c || !o || o->n_steps <= 0 || s0 < 0 || s1 > o->n_steps || s0 > s1 || o->newton_max_it < 1)
        return fail(c, IPFEM_INVALID, "bad Newton options");
    c->ns = NewtonState();
    c->ns.opts = *o;
    c->ns.step = s0;
    c->ns.step_end = s1;
    c->ns.active = 1;
    if (!c->ev_ready) {
        CK(cudaEventCreate(&c->ev[0]));
        CK(cudaEventCreate(&c->ev[1]));
        c->ev_ready = true;
    }
    return IPFEM_OK;
}

ipfem_status ipfem_newton_advance(ipfem_ctx *c, int32_t n_iters, double *u, int where, ipfem_solve_stats *stats,
                                  double *log, int32_t log_cap, int32_t *n_done)
{
    if (!c || !u || n_iters < 0 || (where != IPFEM_HOST && where != IPFEM_DEVICE))
        return fail(c, IPFEM_INVALID, "bad args");
    if (!c->ns.active) return fail(c, IPFEM_INVALID, "ipfem_newton_begin not called");
    const size_t nb = (size_t)c->s.neq * sizeof(double);
    double *du = u;
    if (where == IPFEM_HOST) {
        CK(cudaMemcpyAsync(c->d_u, u, nb, cudaMemcpyHostToDevice, c->stream));
        du = c->d_u;
    }
    ipfem_solve_stats st{};
    int32_t nlog = 0;
    const int saved_update = c->update_mem;
    c->update_mem = 0;
    ipfem_status ret = newton_advance(c, n_iters == 0 ? INT32_MAX : n_iters, du, &st, log, log_cap, &nlog);
    c->update_mem = saved_update;
    if (where == IPFEM_HOST) {
        CK(cudaMemcpyAsync(u, c->d_u, nb, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
    }
    if (stats) *stats = st;
    if (n_done) *n_done = st.newton_iters;
    return ret;
}

ipfem_status ipfem_newton_solve(ipfem_ctx *c, const ipfem_solve_opts *o, int32_t s0, int32_t s1, double *u, int where,
                                ipfem_solve_stats *stats, double *log, int32_t log_cap)
{
    ipfem_status st = ipfem_newton_begin(c, o, s0, s1);
    if (st != IPFEM_OK) return st;
    st = ipfem_newton_advance(c, 0, u, where, stats, log, log_cap, nullptr);
    c->ns.active = 0;
    if (st == IPFEM_OK && stats && !stats->converged)
        return fail(c, IPFEM_NONCONVERGED, "Newton did not converge in every step");
    return st;
}

uint64_t ipfem_launch_count(const ipfem_ctx *c)
{
    return c ? c->launches : 0;
}

ipfem_status ipfem_set_iteration_log(ipfem_ctx *c, const char *path)
{
    if (!c) return IPFEM_INVALID;
    if (c->iter_log) {
        std::fclose(c->iter_log);
        c->iter_log = nullptr;
    }
    if (!path || !*path) return IPFEM_OK;
    c->iter_log = std::fopen(path, "a");
    if (!c->iter_log) return fail(c, IPFEM_INVALID, std::string("cannot open the iteration log ") + path);
    return IPFEM_OK;
}

ipfem_status ipfem_dot(ipfem_ctx *c, const double *d_a, const double *d_b, double *out)
{
    if (!c || !d_a || !d_b || !out) return fail(c, IPFEM_INVALID, "bad args");
    // the dot kernel reads node pairs as 16-byte loads
    if ((reinterpret_cast<uintptr_t>(d_a) | reinterpret_cast<uintptr_t>(d_b)) & 15u)
        return fail(c, IPFEM_INVALID, "ipfem_dot: d_a and d_b must be 16-byte aligned");
    return dot_host(c, d_a, d_b, out);
}

ipfem_status ipfem_measure_fp64_peak(ipfem_ctx *c, double *tflops)
{
    if (!c || !tflops) return fail(c, IPFEM_INVALID, "bad args");
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
    const int grid = sms * 8, iters = 4096;
    double *d = nullptr;
    CK(cudaMallocAsync((void **)&d, (size_t)grid * 256 * sizeof(double), c->stream));
    if (!c->ev_ready) {
        CK(cudaEventCreate(&c->ev[0]));
        CK(cudaEventCreate(&c->ev[1]));
        c->ev_ready = true;
    }
    launch_fp64_probe(c, d, grid, iters);
    CK(cudaEventRecord(c->ev[0], c->stream));
    launch_fp64_probe(c, d, grid, iters);
    CK(cudaEventRecord(c->ev[1], c->stream));
    CK(cudaEventSynchronize(c->ev[1]));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
    CK(cudaFreeAsync(d, c->stream));
    c->launches += 2;
    *tflops = 2.0 * 8.0 * iters * (double)grid * 256 / (ms * 1e-3) / 1e12;
    return sync_check(c);
}

ipfem_status ipfem_profile_spmv(ipfem_ctx *c, int reps, double *ms_per_launch)
{
    if (!c || reps < 1 || !ms_per_launch) return fail(c, IPFEM_INVALID, "bad args");
    if (!c->tangent_valid) return fail(c, IPFEM_INVALID, "no tangent assembled");
    if (!c->ev_ready) {
        CK(cudaEventCreate(&c->ev[0]));
        CK(cudaEventCreate(&c->ev[1]));
        c->ev_ready = true;
    }
    const bool mixed = c->precision == 1;
    if (mixed) {
        launch_cg32_init(c, c->d_rhs, 1.0, 0.0f, 1 << 30);
        launch_cg32_spmv_only(c);
    } else {
        launch_cg_init(c, c->d_rhs, 0.0, 1 << 30);
        launch_cg_spmv_only(c);
    }
    CK(cudaEventRecord(c->ev[0], c->stream));
    for (int k = 0; k < reps; k++) {
        if (mixed) launch_cg32_spmv_only(c);
        else launch_cg_spmv_only(c);
    }
    CK(cudaEventRecord(c->ev[1], c->stream));
    c->launches += 2 + reps;
    CK(cudaEventSynchronize(c->ev[1]));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
    *ms_per_launch = ms / reps;
    return sync_check(c);
}

ipfem_status ipfem_profile_residual(ipfem_ctx *c, const double *d_u, int bits, int reps, double *ms)
{
    if (!c || !d_u || reps < 1 || !ms || (bits != 32 && bits != 64)) return fail(c, IPFEM_INVALID, "bad args");
    if (bits == 32 && (c->precision != IPFEM_MIXED || !c->mx.strain32))
        return fail(c, IPFEM_INVALID, "the FP32 residual kernels need IPFEM_MIXED and "
                                      "ipfem_set_residual_precision(ctx, 32, ...)");
    cudaEvent_t ev[5] = {};
    for (int k = 0; k < 5; k++) {
        const cudaError_t e = cudaEventCreate(&ev[k]);
        if (e != cudaSuccess) {
            for (int j = 0; j < k; j++) cudaEventDestroy(ev[j]);
            return fail(c, IPFEM_CUDA, cudaGetErrorString(e));
        }
    }
    MixedBuffers &m = c->mx;
    double acc[4] = {0, 0, 0, 0};
    cudaError_t e = cudaSuccess;
    for (int r = 0; r < reps && e == cudaSuccess; r++) {
        cudaEventRecord(ev[0], c->stream);
        if (bits == 32) launch_gather_strain32(c, d_u, m.strain32);
        else launch_gather_strain(c, d_u, c->d_strain);
        cudaEventRecord(ev[1], c->stream);
        if (bits == 32) launch_compute_sigma32(c, 0, m.strain32, m.sigw32, nullptr);
        else launch_compute_sigma(c, 0, c->d_strain, c->d_sigma_w, nullptr);
        cudaEventRecord(ev[2], c->stream);
        if (bits == 32) launch_stress_residual32(c, m.sigw32, m.fe32);
        else launch_stress_residual(c, c->d_sigma_w, c->d_fe);
        cudaEventRecord(ev[3], c->stream);
        // into d_b, a scratch vector: d_rhs holds the Newton loop's residual
        if (bits == 32) launch_color_reduce32(c, m.fe32, 1, c->d_b);
        else launch_color_reduce(c, c->d_fe, 1, c->d_b);
        cudaEventRecord(ev[4], c->stream);
        c->launches += 4;
        e = cudaEventSynchronize(ev[4]);
        for (int k = 0; k < 4 && e == cudaSuccess; k++) {
            float t = 0.0f;
            e = cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
            acc[k] += t;
        }
    }
    for (int k = 0; k < 5; k++) cudaEventDestroy(ev[k]);
    if (e != cudaSuccess) return fail(c, IPFEM_CUDA, cudaGetErrorString(e));
    for (int k = 0; k < 4; k++) ms[k] = acc[k] / reps;
    return sync_check(c);
}

ipfem_status ipfem_gather_strain(ipfem_ctx *c, const double *d_u, double *d_strain)
{
    if (!c || !d_u || !d_strain) return fail(c, IPFEM_INVALID, "bad args");
    launch_gather_strain(c, d_u, d_strain);
    return sync_check(c);
}

ipfem_status ipfem_compute_sigma(ipfem_ctx *c, int update_mem, const double *d_strain, double *d_sigma_w,
                                 double *d_dep)
{
    if (!c || !d_strain || !d_sigma_w) return fail(c, IPFEM_INVALID, "bad args");
    launch_compute_sigma(c, update_mem, d_strain, d_sigma_w, d_dep);
    return sync_check(c);
}

ipfem_status ipfem_scatter_residual(ipfem_ctx *c, const double *d_sigma_w, double *d_res)
{
    if (!c || !d_sigma_w || !d_res) return fail(c, IPFEM_INVALID, "bad args");
    launch_stress_residual(c, d_sigma_w, c->d_fe);
    launch_color_reduce(c, c->d_fe, 0, d_res);
    return sync_check(c);
}

ipfem_status ipfem_gather_strain32(ipfem_ctx *c, const double *d_u, float *d_strain)
{
    if (!c || !d_u || !d_strain) return fail(c, IPFEM_INVALID, "bad args");
    if (!c->mx.dphiT) return fail(c, IPFEM_INVALID, "the FP32 residual kernels need ipfem_set_residual_precision(ctx, 32, ...)");
    launch_gather_strain32(c, d_u, d_strain);
    return sync_check(c);
}

ipfem_status ipfem_scatter_residual32(ipfem_ctx *c, const float *d_sigma_w, double *d_res)
{
    if (!c || !d_sigma_w || !d_res) return fail(c, IPFEM_INVALID, "bad args");
    if (!c->mx.dphiT) return fail(c, IPFEM_INVALID, "the FP32 residual kernels need ipfem_set_residual_precision(ctx, 32, ...)");
    launch_stress_residual32(c, d_sigma_w, c->mx.fe32);
    launch_color_reduce32(c, c->mx.fe32, 0, d_res);
    return sync_check(c);
}

ipfem_status ipfem_get_state(ipfem_ctx *c, int field, double *out)
{
    if (!c || !out) return IPFEM_INVALID;
    const int64_t n = c->s.n_ip;
    switch (field) {
    case 0: CK(cudaMemcpyAsync(out, c->d_eps_p, 4 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream)); break;
    case 1: CK(cudaMemcpyAsync(out, c->d_sigma, 4 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream)); break;
    case 2: CK(cudaMemcpyAsync(out, c->d_alpha, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream)); break;
    case 3: {
        std::vector<int8_t> h((size_t)n);
        CK(cudaMemcpyAsync(h.data(), c->d_mtype, (size_t)n, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        for (int64_t i = 0; i < n; i++) out[i] = h[i];
        return IPFEM_OK;
    }
    default: return fail(c, IPFEM_INVALID, "bad state field");
    }
    CK(cudaStreamSynchronize(c->stream));
    return IPFEM_OK;
}

ipfem_status ipfem_set_state(ipfem_ctx *c, int field, const double *in)
{
    if (!c || !in) return IPFEM_INVALID;
    const int64_t n = c->s.n_ip;
    switch (field) {
    case 0: CK(cudaMemcpyAsync(c->d_eps_p, in, 4 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream)); break;
    case 1: CK(cudaMemcpyAsync(c->d_sigma, in, 4 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream)); break;
    case 2: CK(cudaMemcpyAsync(c->d_alpha, in, n * sizeof(double), cudaMemcpyHostToDevice, c->stream)); break;
    case 3: {
        // m_type as double (0 elastic, 1 plane or edge, -1 apex) -> int8
        std::vector<int8_t> h((size_t)n);
        for (int64_t k = 0; k < n; k++) {
            if (!(in[k] == 0.0 || in[k] == 1.0 || in[k] == -1.0))
                return fail(c, IPFEM_INVALID, "m_type values must be 0, 1 or -1");
            h[(size_t)k] = (int8_t)in[k];
        }
        CK(cudaMemcpyAsync(c->d_mtype, h.data(), (size_t)n, cudaMemcpyHostToDevice, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        return IPFEM_OK;
    }
    default: return fail(c, IPFEM_INVALID, "bad state field");
    }
    CK(cudaStreamSynchronize(c->stream));
    return IPFEM_OK;
}

ipfem_status ipfem_get_setup(ipfem_ctx *c, int field, void *out)
{
    if (!c || !out) return IPFEM_INVALID;
    const Setup &s = c->s;
    switch (field) {
    case 0: std::memcpy(out, s.el_color.data(), s.el_color.size() * sizeof(int32_t)); break;
    case 1: *(int32_t *)out = s.n_colors; break;
    case 2: std::memcpy(out, s.dofs.data(), s.dofs.size() * sizeof(int32_t)); break;
    case 3: std::memcpy(out, s.dphi.data(), s.dphi.size() * sizeof(double)); break;
    case 4: std::memcpy(out, s.weight.data(), s.weight.size() * sizeof(double)); break;
    default: return fail(c, IPFEM_INVALID, "bad setup field");
    }
    return IPFEM_OK;
}

}  // extern "C"
