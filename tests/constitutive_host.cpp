// Host build of the device's per-point constitutive update
// (intpointsfem_gb300/csrc/constitutive.cuh) for a CPU test that compares it
// with the oracle bit for bit.  Compiled by tests/test_constitutive_host_cpu.py
// with g++ -ffp-contract=off, the host counterpart of the device's --fmad=false.
#include "../intpointsfem_gb300/csrc/constitutive.cuh"

extern "C" int host_ip_update(int dep, int consistent, int spectral, double lambda, double mu, const double mc5[5],
                              const double eps[3], const double pl[4], double weight, double sigma_w3[3],
                              double sig4[4], double pl_out4[4], double *alpha, double dep9[9])
{
    // the elastic constants as the library's setup forms them (host_setup.cpp)
    ElasticConst E;
    E.lambda = lambda;
    E.mu = mu;
    E.K = lambda + 2 * mu / 3;
    E.G = mu;
    E.l2m = lambda + 2 * mu;
    E.c1 = (lambda + mu) / (3 * lambda * mu + 2 * mu * mu);
    E.c2 = lambda / (6 * lambda * mu + 4 * mu * mu);
    E.inv_mu = 1 / mu;
    E.consistent = consistent;
    E.spectral = spectral;
    MCConst m;
    m.c = mc5[0];
    m.sinphi = mc5[1];
    m.cosphi = mc5[2];
    m.tanphi = mc5[3];
    m.sinpsi = mc5[4];
    double a = 0.0, d[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int mt = dep ? ip_update<true>(eps, pl, E, m, sig4, pl_out4, a, d)
                       : ip_update<false>(eps, pl, E, m, sig4, pl_out4, a, d);
    // the kernel's weighting (k_compute_sigma)
    sigma_w3[0] = sig4[0] * weight;
    sigma_w3[1] = sig4[1] * weight;
    sigma_w3[2] = sig4[2] * weight;
    if (dep)
        for (int k = 0; k < 9; k++) dep9[k] = d[k] * weight;
    *alpha = a;
    return mt;
}
