// Drives ipfem::pz::TPZElastoPlasticIntPointsStructMatrix the way the
// reference's analysis drives its struct matrix (main.cpp:280-285, 487-522):
// construct, Assemble(rhs), CreateAssemble(rhs), Clone() and Assemble(rhs) on
// the clone, a state commit through SetUpdateMem, and the error path.
//
//   struct_matrix_driver <n> <lambda> <dir>
//
// builds the n x n wellbore problem, reads the displacement from <dir>/u.bin
// (neq doubles; zeros when absent) and writes res.bin, rhs_k.bin, ia.bin,
// ja.bin, a.bin, pattern_ja.bin, clone_res.bin, res_after_commit.bin into
// <dir>.  A std::runtime_error ends the program with "runtime_error: <what>"
// and exit code 3 (no device: the constructor throws).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "ipfem_pz.hpp"

using ipfem::pz::SymSparse;
using ipfem::pz::TPZElastoPlasticIntPointsStructMatrix;

template <class T>
static void write(const std::string &path, const std::vector<T> &v)
{
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f || std::fwrite(v.data(), sizeof(T), v.size(), f) != v.size()) {
        std::fprintf(stderr, "cannot write %s\n", path.c_str());
        std::exit(2);
    }
    std::fclose(f);
}

static bool read(const std::string &path, std::vector<double> &v)
{
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    const size_t n = std::fread(v.data(), sizeof(double), v.size(), f);
    std::fclose(f);
    return n == v.size();
}

int main(int argc, char **argv)
{
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s n lambda dir\n", argv[0]);
        return 2;
    }
    const int n = std::atoi(argv[1]);
    const double lam = std::atof(argv[2]);
    const std::string dir = argv[3];
    ipfem_wellbore_params prm;
    ipfem_wellbore_default(&prm, n);
    ipfem_wellbore *wb = nullptr;
    if (ipfem_wellbore_build(&prm, &wb) != IPFEM_OK) {
        std::fprintf(stderr, "wellbore build failed\n");
        return 2;
    }
    try {
        // the element order of a mesh the class refuses
        bool refused = false;
        try {
            ipfem_mesh bad = wb->mesh;
            bad.order = 7;
            TPZElastoPlasticIntPointsStructMatrix x(bad, wb->material);
        } catch (const std::runtime_error &) {
            refused = true;
        }
        if (!refused) {
            std::fprintf(stderr, "order 7 was accepted\n");
            return 1;
        }
        TPZElastoPlasticIntPointsStructMatrix sm(wb->mesh, wb->material);
        ipfem_wellbore_free(wb);   // the object keeps its own copy of the problem
        wb = nullptr;
        std::vector<double> &u = sm.Solution();
        read(dir + "/u.bin", u);
        sm.SetLoadFactor(lam);
        std::vector<double> res;
        sm.Assemble(res);
        write(dir + "/res.bin", res);
        SymSparse *pattern = sm.Create();
        write(dir + "/pattern_ja.bin", pattern->JA);
        for (double v : pattern->A)
            if (v != 0.0) {
                std::fprintf(stderr, "Create() returned non-zero values\n");
                return 1;
            }
        delete pattern;
        std::vector<double> rhs;
        SymSparse *K = sm.CreateAssemble(rhs);
        write(dir + "/rhs_k.bin", rhs);
        write(dir + "/ia.bin", K->IA);
        write(dir + "/ja.bin", K->JA);
        write(dir + "/a.bin", K->A);
        if (K->GetVal(0, 1) != K->GetVal(1, 0)) return 1;
        delete K;
        // Clone: same problem, load factor, solution and state
        TPZElastoPlasticIntPointsStructMatrix *cl = sm.Clone();
        std::vector<double> res_c;
        cl->Assemble(res_c);
        write(dir + "/clone_res.bin", res_c);
        delete cl;
        // commit the state at u, then the residual of the next evaluation
        sm.SetUpdateMem(true);
        sm.Assemble(res);
        sm.SetUpdateMem(false);
        sm.Assemble(res);
        write(dir + "/res_after_commit.bin", res);
        // errors throw with the library's message
        try {
            sm.SetLoadFactor(NAN);
            std::fprintf(stderr, "a NaN load factor was accepted\n");
            return 1;
        } catch (const std::runtime_error &e) {
            std::printf("error path: %s\n", e.what());
        }
    } catch (const std::runtime_error &e) {
        std::printf("runtime_error: %s\n", e.what());
        if (wb) ipfem_wellbore_free(wb);
        return 3;
    }
    std::printf("ok\n");
    return 0;
}
