// Integration-point constitutive kernels: one integration point per thread,
// FP64, structure-of-arrays state (TPZCudaCalls::ComputeSigma /
// ComputeSigmaDep and KernelsComputeSigma.h of the reference, CPU-path
// semantics).  Compiled with --fmad=false: see constitutive.cuh.
#include "ipfem_internal.h"
#include "constitutive.cuh"

namespace ipfem {

// TS = double: the plain path; TS = float: the FP32 strain and weighted
// stress arrays of the mixed-precision residual (the point update itself
// stays FP64: the strain is widened, the weighted stress rounded at the end).
template <bool DEP, bool UPD, class TS>
__global__ void __launch_bounds__(128) k_compute_sigma(int64_t n_ip, int32_t n_el, int32_t npts, ElasticConst E,
                                                       const TS *__restrict__ strain,
                                                       const double *__restrict__ weight,
                                                       const double *__restrict__ mat,
                                                       double *__restrict__ eps_p,
                                                       TS *__restrict__ sigma_w,
                                                       double *__restrict__ dep,
                                                       double *__restrict__ sig_state,
                                                       int8_t *__restrict__ mtype,
                                                       double *__restrict__ alpha_state)
{
    const int64_t ip = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (ip >= n_ip) return;
    const int64_t e = ip / npts;
    MCConst m;
    m.c = __ldg(&mat[e]);
    m.sinphi = __ldg(&mat[n_el + e]);
    m.cosphi = __ldg(&mat[2 * (int64_t)n_el + e]);
    m.tanphi = __ldg(&mat[3 * (int64_t)n_el + e]);
    m.sinpsi = __ldg(&mat[4 * (int64_t)n_el + e]);
    const double eps[3] = {(double)strain[ip], (double)strain[n_ip + ip], (double)strain[2 * n_ip + ip]};
    const double pl[4] = {eps_p[ip], eps_p[n_ip + ip], eps_p[2 * n_ip + ip], eps_p[3 * n_ip + ip]};
    double sig[4], plo[4], a, d[9];
    const int mt = ip_update<DEP>(eps, pl, E, m, sig, plo, a, d);
    const double w = weight[ip];
    sigma_w[ip] = (TS)(sig[0] * w);
    sigma_w[n_ip + ip] = (TS)(sig[1] * w);
    sigma_w[2 * n_ip + ip] = (TS)(sig[2] * w);
    if (DEP) {
#pragma unroll
        for (int k = 0; k < 9; k++) dep[k * n_ip + ip] = d[k] * w;
    }
    if (UPD) {
#pragma unroll
        for (int k = 0; k < 4; k++) {
            eps_p[k * n_ip + ip] = plo[k];
            sig_state[k * n_ip + ip] = sig[k];
        }
        mtype[ip] = (int8_t)mt;
        alpha_state[ip] = a;
    }
}

template <class TS>
static void compute_sigma_t(ipfem_ctx *c, int update_mem, const TS *d_strain, TS *d_sigma_w, double *d_dep)
{
    const Setup &s = c->s;
    ElasticConst E;
    E.lambda = s.el.lambda; E.mu = s.el.mu; E.K = s.el.K; E.G = s.el.G; E.l2m = s.el.l2m;
    E.c1 = s.el.c1; E.c2 = s.el.c2; E.inv_mu = s.el.inv_mu;
    E.consistent = c->consistent_tangent;
    E.spectral = c->spectral_mode;
    const int tpb = 128;
    const unsigned grid = (unsigned)((s.n_ip + tpb - 1) / tpb);
    if (grid == 0) return;
#define ARGS s.n_ip, s.n_el, s.nq, E, d_strain, c->d_weight, c->d_mat, c->d_eps_p, d_sigma_w, d_dep, c->d_sigma, \
             c->d_mtype, c->d_alpha
    if (d_dep) {
        if (update_mem) k_compute_sigma<true, true, TS><<<grid, tpb, 0, c->stream>>>(ARGS);
        else k_compute_sigma<true, false, TS><<<grid, tpb, 0, c->stream>>>(ARGS);
    } else {
        if (update_mem) k_compute_sigma<false, true, TS><<<grid, tpb, 0, c->stream>>>(ARGS);
        else k_compute_sigma<false, false, TS><<<grid, tpb, 0, c->stream>>>(ARGS);
    }
#undef ARGS
}

void launch_compute_sigma(ipfem_ctx *c, int update_mem, const double *d_strain, double *d_sigma_w, double *d_dep)
{
    compute_sigma_t<double>(c, update_mem, d_strain, d_sigma_w, d_dep);
}

void launch_compute_sigma32(ipfem_ctx *c, int update_mem, const float *d_strain, float *d_sigma_w, double *d_dep)
{
    compute_sigma_t<float>(c, update_mem, d_strain, d_sigma_w, d_dep);
}

}  // namespace ipfem
