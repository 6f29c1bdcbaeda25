// ipfem_pz.hpp -- C++ face of libipfem with the reference's struct-matrix API.
//
// The reference's NeoPZ analysis drives its integration-point path through
// TPZElastoPlasticIntPointsStructMatrix (TPZElastoPlasticIntPointsStructMatrix.h:33-42):
// Create() / CreateAssemble(rhs) once, Assemble(K, rhs) for tangent and
// residual, Assemble(rhs) for the residual alone, Clone(); the displacement is
// read from the mesh's Solution(), the state commit is switched by the
// material's SetUpdateMem (main.cpp:499, 514), and every failure throws
// std::runtime_error (TPZCudaCalls.cu:42-49).  This header-only class keeps
// those names and that behaviour over the C-ABI of ipfem.h: one ipfem context
// per object (device buffers and stream), released by the destructor.
//
// Matrices are SymSparse: the upper triangle (column >= row) of the dof
// matrix in CSR with int64 indices, the layout of NeoPZ's TPZSYsmpMatrix
// (IA, JA, A) that the reference's colour-ordered assembly writes
// (TPZNumericalIntegrator.cpp:538-606).  Vectors are std::vector<double> of
// length NEquations().
#ifndef IPFEM_PZ_HPP
#define IPFEM_PZ_HPP

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "ipfem.h"

namespace ipfem {
namespace pz {

// TPZSYsmpMatrix's storage: IA[neq+1], JA[nnz], A[nnz], upper triangle
struct SymSparse {
    int64_t neq = 0;
    std::vector<int64_t> IA, JA;
    std::vector<double> A;
    // A(row, col) for any row, col (mirrored below the diagonal; 0 off the pattern)
    double GetVal(int64_t row, int64_t col) const
    {
        if (row > col) std::swap(row, col);
        for (int64_t k = IA[row]; k < IA[row + 1]; k++)
            if (JA[k] == col) return A[k];
        return 0.0;
    }
};

// Owned copy of a problem description: ipfem_create reads its arrays only
// while it runs, and Clone() builds a second context from the same data.
class MeshData {
public:
    MeshData(const ipfem_mesh &m, const ipfem_material &mat) : mesh_(m), mat_(mat)
    {
        if (m.n_elements <= 0 || m.n_nodes <= 0 || !m.connects || !m.weight || (!m.dphi && !m.block_storage))
            throw std::runtime_error("ipfem: incomplete mesh description");
        const int order = m.order ? m.order : 2;
        if (order < 1 || order > IPFEM_MAX_ORDER) throw std::runtime_error("ipfem: element order must be 1, 2 or 3");
        const size_t nn = (size_t)(order + 1) * (order + 1), ne = (size_t)m.n_elements, neq = 2 * (size_t)m.n_nodes;
        copy(connects_, m.connects, ne * nn);
        copy(dphi_, m.dphi, ne * nn * 2 * nn);
        copy(storage_, m.block_storage, ne * (3 * nn) * (2 * nn));
        copy(weight_, m.weight, ne * nn);
        copy(fixed_, m.fixed, neq);
        copy(f0_, m.f0, neq);
        copy(df_, m.df, neq);
        copy(el_c_, mat.el_cohesion, ne);
        copy(el_phi_, mat.el_phi, ne);
        mesh_.connects = connects_.empty() ? nullptr : connects_.data();
        mesh_.dphi = dphi_.empty() ? nullptr : dphi_.data();
        mesh_.block_storage = storage_.empty() ? nullptr : storage_.data();
        mesh_.weight = weight_.empty() ? nullptr : weight_.data();
        mesh_.fixed = fixed_.empty() ? nullptr : fixed_.data();
        mesh_.f0 = f0_.empty() ? nullptr : f0_.data();
        mesh_.df = df_.empty() ? nullptr : df_.data();
        mat_.el_cohesion = el_c_.empty() ? nullptr : el_c_.data();
        mat_.el_phi = el_phi_.empty() ? nullptr : el_phi_.data();
    }
    const ipfem_mesh &mesh() const { return mesh_; }
    const ipfem_material &material() const { return mat_; }

private:
    template <class T>
    static void copy(std::vector<T> &dst, const T *src, size_t n)
    {
        if (src) dst.assign(src, src + n);
    }
    ipfem_mesh mesh_;
    ipfem_material mat_;
    std::vector<int32_t> connects_;
    std::vector<double> dphi_, storage_, weight_, f0_, df_, el_c_, el_phi_;
    std::vector<uint8_t> fixed_;
};

class TPZElastoPlasticIntPointsStructMatrix {
public:
    // the reference constructs from a TPZCompMesh*; here from the mesh
    // description that SetUpDataStructure extracts from it
    // (TPZElastoPlasticIntPointsStructMatrix.cpp:80-97)
    TPZElastoPlasticIntPointsStructMatrix(const ipfem_mesh &mesh, const ipfem_material &mat)
        : data_(std::make_shared<MeshData>(mesh, mat))
    {
        open();
    }
    // copy construction is Clone() (TPZElastoPlasticIntPointsStructMatrix.cpp:30-32):
    // a new context on the same problem data, with the source's load factor,
    // solution and integration-point state (the reference copies its
    // integrator, whose constitutive processor holds that state)
    TPZElastoPlasticIntPointsStructMatrix(const TPZElastoPlasticIntPointsStructMatrix &o)
        : data_(o.data_), solution_(o.solution_), load_factor_(o.load_factor_)
    {
        open();
        Check(ipfem_set_load_factor(ctx_, load_factor_));
        int64_t sz[6];
        Check(ipfem_sizes(ctx_, sz));
        std::vector<double> f;
        for (int field = 0; field < 4; field++) {
            f.resize((size_t)(field < 2 ? 4 : 1) * (size_t)sz[1]);
            o.Check(ipfem_get_state(o.ctx_, field, f.data()));
            Check(ipfem_set_state(ctx_, field, f.data()));
        }
    }
    TPZElastoPlasticIntPointsStructMatrix &operator=(const TPZElastoPlasticIntPointsStructMatrix &) = delete;
    ~TPZElastoPlasticIntPointsStructMatrix()
    {
        if (ctx_) ipfem_destroy(ctx_);
    }

    TPZElastoPlasticIntPointsStructMatrix *Clone() const { return new TPZElastoPlasticIntPointsStructMatrix(*this); }

    // TPZSYsmpMatrix with the tangent's pattern, values zero
    // (TPZElastoPlasticIntPointsStructMatrix.cpp:34-60)
    SymSparse *Create()
    {
        std::unique_ptr<SymSparse> K(new SymSparse);
        Export(*K, false);
        return K.release();
    }

    // Create() followed by Assemble(K, rhs) (TPZElastoPlasticIntPointsStructMatrix.cpp:71-78)
    SymSparse *CreateAssemble(std::vector<double> &rhs)
    {
        std::unique_ptr<SymSparse> K(Create());
        Assemble(*K, rhs);
        return K.release();
    }

    // tangent and residual at Solution() (TPZElastoPlasticIntPointsStructMatrix.cpp:99-135):
    // rhs = -B^T sigma(u) + rhs_linear, K the tangent: the reference's
    // TangentOperator, or the consistent one after
    // ipfem_set_consistent_tangent(Context(), 1)
    void Assemble(SymSparse &K, std::vector<double> &rhs)
    {
        rhs.assign((size_t)NEquations(), 0.0);
        Check(ipfem_assemble(ctx_, solution_.data(), rhs.data(), IPFEM_HOST));
        Export(K);
    }

    // residual only at Solution() (TPZElastoPlasticIntPointsStructMatrix.cpp:137-154)
    void Assemble(std::vector<double> &rhs)
    {
        rhs.assign((size_t)NEquations(), 0.0);
        Check(ipfem_assemble_residual(ctx_, solution_.data(), rhs.data(), IPFEM_HOST));
    }

    // the displacement the assemblies read (the reference's fMesh->Solution())
    std::vector<double> &Solution() { return solution_; }
    // TPZMatWithMem::SetUpdateMem: the next residual commits the point state
    void SetUpdateMem(bool update) { Check(ipfem_set_update_mem(ctx_, update ? 1 : 0)); }
    // rhs_linear = f0 + lambda df (the reference's fRhsLinear)
    void SetLoadFactor(double lambda)
    {
        Check(ipfem_set_load_factor(ctx_, lambda));
        load_factor_ = lambda;
    }
    int64_t NEquations() const { return neq_; }
    ipfem_ctx *Context() { return ctx_; }

    // throws std::runtime_error with the context's message, as the reference's
    // TPZCudaCalls does after every failed call (TPZCudaCalls.cu:42-49)
    void Check(ipfem_status st) const
    {
        if (st != IPFEM_OK)
            throw std::runtime_error(std::string("ipfem: ") + ipfem_status_string(st) + ": " +
                                     ipfem_last_error(ctx_));
    }

private:
    void open()
    {
        const ipfem_status st = ipfem_create(&data_->mesh(), &data_->material(), &ctx_);
        if (st != IPFEM_OK) {
            ctx_ = nullptr;
            throw std::runtime_error(std::string("ipfem: ") + ipfem_status_string(st) + ": " +
                                     ipfem_last_error(nullptr));
        }
        int64_t sz[6];
        Check(ipfem_sizes(ctx_, sz));
        neq_ = sz[3];
        if ((int64_t)solution_.size() != neq_) solution_.assign((size_t)neq_, 0.0);
    }

    void Export(SymSparse &K, bool values = true)
    {
        int64_t nnz = 0;
        Check(ipfem_get_stiffness_sym_csr(ctx_, &nnz, nullptr, nullptr, nullptr));
        K.neq = neq_;
        K.IA.resize((size_t)neq_ + 1);
        K.JA.resize((size_t)nnz);
        K.A.assign((size_t)nnz, 0.0);
        Check(ipfem_get_stiffness_sym_csr(ctx_, &nnz, K.IA.data(), K.JA.data(), values ? K.A.data() : nullptr));
    }

    std::shared_ptr<MeshData> data_;
    ipfem_ctx *ctx_ = nullptr;
    std::vector<double> solution_;
    int64_t neq_ = 0;
    double load_factor_ = 0.0;
};

}  // namespace pz
}  // namespace ipfem

#endif  // IPFEM_PZ_HPP
