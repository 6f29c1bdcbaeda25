/*
 * Test infrastructure: drives the reference's own constitutive functions
 * (FunctionsStressStrain.h, FunctionsTangentOperator.h and the two headers
 * they include, compiled unmodified from the reference tree) through the
 * per-point sequences of the reference, to produce golden vectors.
 *
 *  ref_ip_sigma      : TPZConstitutiveLawProcessor.cpp:163-195 (CPU ComputeSigma)
 *  ref_ip_sigma_dep  : TPZConstitutiveLawProcessor.cpp:377-423 (CPU ComputeSigmaDep)
 *  ref_ip_sigma_gpu  : KernelsComputeSigma.h:7-74 (GPU ComputeSigmaKernel,
 *                      whose ProjectSigma call aliases input and output)
 *
 * Built by oracle/build.py into oracle/_ref/ only; never part of the product.
 */
#include "FunctionsStressStrain.h"
#include "FunctionsTangentOperator.h"

extern "C" {

void ref_ip_sigma(double lambda, double mu, double phi, double psi, double c,
                  const double *delta_strain3, const double *plastic6, double weight,
                  double *sigma_w3, double *sigma6, double *plastic6_out,
                  int *mtype, double *alpha)
{
    REAL G = mu, K = lambda + 2 * mu / 3;
    REAL aux[3] = {delta_strain3[0], delta_strain3[1], delta_strain3[2]};
    REAL strain[6] = {0, 0, 0, 0, 0, 0}, ee[6], sig[6], pl[6];
    REAL sev[3] = {0, 0, 0}, svec[9] = {0}, sp[3] = {0, 0, 0}, grad[9] = {0};
    REAL a = 0.0;
    int mt = 0;
    ComposeStrain(aux, strain);
    for (int i = 0; i < 6; i++) pl[i] = plastic6[i];
    ElasticStrain(pl, strain, ee);
    ComputeTrialStress(ee, sig, mu, lambda);
    SpectralDecomposition(sig, sev, svec);
    ProjectSigma(sev, sp, mt, a, phi, psi, c, K, G, grad, false);
    ReconstructStressTensor(sp, svec, sig);
    ComputeStrain(sig, ee, mu, lambda);
    PlasticStrain(strain, ee, pl);
    TranslateStress(sig, aux);
    for (int i = 0; i < 3; i++) sigma_w3[i] = aux[i] * weight;
    for (int i = 0; i < 6; i++) { sigma6[i] = sig[i]; plastic6_out[i] = pl[i]; }
    *mtype = mt;
    *alpha = a;
}

void ref_ip_sigma_dep(double lambda, double mu, double phi, double psi, double c,
                      const double *delta_strain3, const double *plastic6, double weight,
                      double *sigma_w3, double *dep9, double *sigma6, double *plastic6_out,
                      int *mtype, double *alpha)
{
    REAL G = mu, K = lambda + 2 * mu / 3;
    REAL aux[3] = {delta_strain3[0], delta_strain3[1], delta_strain3[2]};
    REAL strain[6] = {0, 0, 0, 0, 0, 0}, ee[6], sig[6], pl[6];
    REAL sev[3] = {0, 0, 0}, svec[9] = {0}, sp[3] = {0, 0, 0}, grad[9] = {0}, dep[36] = {0};
    REAL eev[3] = {0, 0, 0}, evec[9] = {0};
    REAL a = 0.0;
    int mt = 0;
    ComposeStrain(aux, strain);
    for (int i = 0; i < 6; i++) pl[i] = plastic6[i];
    ElasticStrain(pl, strain, ee);
    ComputeTrialStress(ee, sig, mu, lambda);
    SpectralDecomposition(sig, sev, svec);
    ee[1] = ee[1] / 2;
    SpectralDecomposition(ee, eev, evec);
    ProjectSigma(sev, sp, mt, a, phi, psi, c, K, G, grad, true);
    TangentOperator(grad, sev, eev, evec, dep, G, lambda);
    ReconstructStressTensor(sp, svec, sig);
    ComputeStrain(sig, ee, mu, lambda);
    PlasticStrain(strain, ee, pl);
    TranslateStress(sig, aux);
    TranslateDep(dep, grad);
    for (int i = 0; i < 3; i++) sigma_w3[i] = aux[i] * weight;
    for (int i = 0; i < 9; i++) dep9[i] = grad[i] * weight;
    for (int i = 0; i < 6; i++) { sigma6[i] = sig[i]; plastic6_out[i] = pl[i]; }
    *mtype = mt;
    *alpha = a;
}

void ref_ip_sigma_gpu(double lambda, double mu, double phi, double psi, double c,
                      const double *delta_strain3, const double *plastic6, double weight,
                      double *sigma_w3, double *sigma6, double *plastic6_out,
                      int *mtype, double *alpha)
{
    REAL G = mu, K = lambda + 2 * mu / 3;
    REAL aux[3] = {delta_strain3[0], delta_strain3[1], delta_strain3[2]};
    REAL strain[6] = {0, 0, 0, 0, 0, 0}, ee[6], sig[6], pl[6];
    REAL svec[9] = {0}, sp[3] = {0, 0, 0}, grad[9] = {0};
    REAL a = 0.0;
    int mt = 0;
    ComposeStrain(aux, strain);
    for (int i = 0; i < 6; i++) pl[i] = plastic6[i];
    ElasticStrain(pl, strain, ee);
    ComputeTrialStress(ee, sig, mu, lambda);
    SpectralDecomposition(sig, sp, svec);
    ProjectSigma(sp, sp, mt, a, phi, psi, c, K, G, grad, false);
    ReconstructStressTensor(sp, svec, sig);
    ComputeStrain(sig, ee, mu, lambda);
    PlasticStrain(strain, ee, pl);
    TranslateStress(sig, aux);
    for (int i = 0; i < 3; i++) sigma_w3[i] = weight * aux[i];
    for (int i = 0; i < 6; i++) { sigma6[i] = sig[i]; plastic6_out[i] = pl[i]; }
    *mtype = mt;
    *alpha = a;
}

}
