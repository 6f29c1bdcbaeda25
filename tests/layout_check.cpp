// Host-side checks of the block-matrix layouts (no GPU): builds the setup of
// a mesh with the library's own host code (host_setup.cpp, host_gmsh.cpp)
// and verifies, for the FP64 layout (rows sorted by length, one slot per lane
// and block) and the FP32 layout (node order, slot pairs):
//   - every block of every row has one slot inside its slice, no slot twice,
//     the stored column, the block map and the diagonal map agree with the
//     nodal pattern;
//   - with slot pairs, blocks 2j and 2j+1 of a row share one 32-byte sector
//     of 16-byte FP32 blocks;
//   - with row stencils, node + offset gives every block's column.
// It prints one line per layout: name, stencils, slots, and the 32-byte
// sectors an FP32 SpMV touches (lanes with k < row length).
//
//   layout_check wellbore <n>            n x n order-2 wellbore
//   layout_check gmsh <file.msh> <order> Gmsh mesh with the reference's BCs
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <set>
#include <string>
#include <vector>

#include "ipfem_internal.h"

using namespace ipfem;

// the library keeps the last host-side error per thread for ipfem_last_error
// (capi.cpp, which needs the CUDA runtime); here it is printed
namespace ipfem {
void set_thread_error(const std::string &msg) { std::printf("error: %s\n", msg.c_str()); }
}  // namespace ipfem

static int fail(const char *what, int64_t a, int64_t b)
{
    std::printf("FAIL %s %lld %lld\n", what, (long long)a, (long long)b);
    return 1;
}

static int check(const Setup &s, const SellLayout &L, const char *name)
{
    std::vector<char> used((size_t)L.n_sell, 0);
    std::set<int64_t> sectors;
    for (int32_t t = 0; t < s.n_nodes; t++) {
        const int32_t i = L.sell_node[t];
        const int64_t len = s.row_ptr[i + 1] - s.row_ptr[i];
        if (L.rowlen[t] != len) return fail("rowlen", t, L.rowlen[t]);
        const int64_t lo = L.slice_base[t / 32], hi = L.slice_base[t / 32 + 1];
        for (int64_t k = 0; k < len; k++) {
            const int64_t slot = sell_slot(L, t, k);
            if (slot < lo || slot >= hi) return fail("slot outside slice", t, k);
            if (used[(size_t)slot]++) return fail("slot used twice", t, k);
            const int32_t c = s.col[(size_t)(s.row_ptr[i] + k)];
            if (L.sell_col[(size_t)slot] != c) return fail("column", t, k);
            if (L.bsr_to_sell[(size_t)(s.row_ptr[i] + k)] != slot) return fail("block map", t, k);
            if (c == i && L.diag_blk[(size_t)i] != slot) return fail("diagonal", t, k);
            if (L.pair && (k & 1) && sell_slot(L, t, k - 1) / 2 != slot / 2) return fail("pair sector", t, k);
            if (L.n_pat > 0) {
                const int32_t off = L.pat_off[(size_t)L.pat_id[(size_t)t] * kPatLen + k];
                if (i + off != c) return fail("stencil", t, k);
            }
            sectors.insert(slot / 2);
        }
    }
    if (L.n_pat > kPatMax) return fail("stencil count", L.n_pat, kPatMax);
    std::printf("%s stencils %d slots %lld sectors %lld\n", name, L.n_pat, (long long)L.n_sell,
                (long long)sectors.size());
    return 0;
}

// the upper-only layout: every stored block, every lower block through its
// stored twin (bsr_to_sell and the transposed stencils), the block map of the
// assembly (-1 for lower pairs) and the diagonal map
static int check_sym(const Setup &s, const SellLayout &L)
{
    std::vector<char> used((size_t)L.n_sell, 0);
    int64_t stored = 0, lower = 0;
    for (int32_t i = 0; i < s.n_nodes; i++) {
        int64_t k_up = 0, k_lo = 0;
        const int tp = L.tpat_id[(size_t)i];
        for (int64_t b = s.row_ptr[i]; b < s.row_ptr[i + 1]; b++) {
            const int32_t c = s.col[(size_t)b];
            const int64_t code = L.bsr_to_sell[(size_t)b];
            if (c >= i) {
                const int64_t slot = sell_slot(L, i, k_up);
                if (code != slot) return fail("sym block map", i, c);
                if (L.sell_col[(size_t)slot] != c) return fail("sym column", i, c);
                if (used[(size_t)slot]++) return fail("sym slot used twice", i, c);
                if (i + L.pat_off[(size_t)L.pat_id[(size_t)i] * kPatLen + k_up] != c) return fail("sym stencil", i, c);
                if (c == i && L.diag_blk[(size_t)i] != slot) return fail("sym diagonal", i, c);
                k_up++;
                stored++;
            } else {
                const int32_t off = L.tpat[((size_t)tp * kPatLen + k_lo) * 2];
                const int32_t q = L.tpat[((size_t)tp * kPatLen + k_lo) * 2 + 1];
                if (i + off != c) return fail("transposed stencil offset", i, c);
                const int64_t twin = sell_slot(L, c, q);
                if (code != -2 - twin) return fail("lower block code", i, c);
                if (L.sell_col[(size_t)twin] != i) return fail("twin column", i, c);
                k_lo++;
                lower++;
            }
        }
        if (k_up != L.rowlen[(size_t)i] || k_lo != L.tpat_len[(size_t)tp]) return fail("sym row length", i, k_up);
    }
    for (int64_t e = 0; e < s.n_el; e++)
        for (int a = 0; a < s.nn; a++)
            for (int b = 0; b < s.nn; b++) {
                const int32_t r = s.dofs[(size_t)e * s.nd + 2 * a] >> 1, c = s.dofs[(size_t)e * s.nd + 2 * b] >> 1;
                const int32_t eb = L.el_blk[((size_t)e * s.nn + a) * s.nn + b];
                if (c < r ? eb != -1 : (eb < 0 || L.sell_col[(size_t)eb] != c)) return fail("sym element map", e, a);
            }
    std::printf("fp32-sym stencils %d slots %lld sectors %lld tstencils %d stored %lld lower %lld\n", L.n_pat,
                (long long)L.n_sell, (long long)((L.n_sell + 1) / 2), L.n_tpat, (long long)stored, (long long)lower);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc < 3) return 2;
    ipfem_wellbore *w = nullptr;
    ipfem_gmsh *g = nullptr;
    if (!std::strcmp(argv[1], "wellbore")) {
        ipfem_wellbore_params p;
        ipfem_wellbore_default(&p, std::atoi(argv[2]));
        if (ipfem_wellbore_build(&p, &w) != IPFEM_OK) return fail("wellbore", 0, 0);
    } else {
        if (argc < 4 || ipfem_gmsh_read(argv[2], &g) != IPFEM_OK) return fail("gmsh read", 0, 0);
        // the reference's boundary conditions: well and far-field pressure, two symmetry points
        ipfem_bc bcs[4];
        std::memset(bcs, 0, sizeof bcs);
        const char *names[4] = {"bc_wellbore", "bc_farfield", "fixed_x", "fixed_y"};
        const int types[4] = {6, 6, 3, 3};
        const double v[4][2] = {{-10.0, 0.0}, {-0.00625, 0.0}, {1.0, 0.0}, {0.0, 1.0}};
        int32_t nb = 0, omega = -1;
        for (int32_t k = 0; k < g->n_phys; k++) {
            if (!std::strcmp(g->phys_name[k], "Omega")) omega = g->phys_tag[k];
            for (int b = 0; b < 4; b++)
                if (!std::strcmp(g->phys_name[k], names[b])) {
                    bcs[nb].phys = g->phys_tag[k];
                    bcs[nb].type = types[b];
                    bcs[nb].val[0] = v[b][0];
                    bcs[nb].val[1] = v[b][1];
                    nb++;
                }
        }
        ipfem_material mat;
        std::memset(&mat, 0, sizeof mat);
        mat.E = 2000.0;
        mat.nu = 0.2;
        mat.cohesion = 5.0;
        mat.phi = 20.0 * 3.14159265358979323846 / 180.0;
        mat.psi = mat.phi;
        if (ipfem_gmsh_problem(g, std::atoi(argv[3]), omega, bcs, nb, &mat, &w) != IPFEM_OK)
            return fail("gmsh problem", 0, 0);
    }
    Setup s;
    const std::string e = build_setup(&w->mesh, &w->material, s);
    if (!e.empty()) {
        std::printf("FAIL setup %s\n", e.c_str());
        return 1;
    }
    int bad = check(s, s.sell, "fp64");
    SellLayout single, pair;
    build_sell(s, false, false, single);
    build_row_stencils(single);
    build_sell(s, false, true, pair);
    build_row_stencils(pair);
    bad |= check(s, single, "fp32-single");
    bad |= check(s, pair, "fp32-pairs");
    SellLayout sym;
    const std::string es = build_sell_sym(s, sym);
    if (es.empty()) bad |= check_sym(s, sym);
    else std::printf("fp32-sym none: %s\n", es.c_str());
    ipfem_wellbore_free(w);
    if (g) ipfem_gmsh_free(g);
    return bad;
}
