// Host-side setup of libipfem: the data structures the reference builds in
// TPZNumericalIntegrator::SetUpIrregularBlocksData / SetUpIndexes /
// SetUpColoredIndexes / FillLIndexes (TPZNumericalIntegrator.cpp:272-590),
// and the quarter-annulus wellbore mesh provider that stands in for the
// reference's NeoPZ/Gmsh mesh (main.cpp:447-464, 542-607).
//
// Compiled with -ffp-contract=off so that every value (coordinates, element
// blocks, weights, loads) is the separately rounded result of the written
// expression on every host architecture.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <new>
#include <thread>

#include "ipfem_internal.h"

namespace ipfem {

void elastic_constants(double E, double nu, ElasticConstH &el)
{
    el.lambda = (E * nu) / ((1.0 + nu) * (1.0 - 2.0 * nu));
    el.mu = E / (2.0 * (1.0 + nu));
    const double lambda = el.lambda, mu = el.mu;
    el.K = lambda + 2 * mu / 3;
    el.G = mu;
    el.l2m = lambda + 2 * mu;
    el.c1 = (lambda + mu) / (3 * lambda * mu + 2 * mu * mu);
    el.c2 = lambda / (6 * lambda * mu + 4 * mu * mu);
    el.inv_mu = 1 / mu;
}

// TPZNumericalIntegrator::SetUpColoredIndexes (TPZNumericalIntegrator.cpp:452-536):
// repeated passes over the elements in index order; an element takes the
// current colour iff none of its connects is marked in this pass.
int32_t greedy_coloring_nn(int32_t n_el, int32_t n_nodes, int32_t nn, const int32_t *connects, int32_t *el_color)
{
    std::vector<uint8_t> mark((size_t)n_nodes, 0);
    std::fill(el_color, el_color + n_el, -1);
    int32_t color = 0;
    bool again = true;
    while (again) {
        again = false;
        for (int32_t e = 0; e < n_el; e++) {
            if (el_color[e] != -1) continue;
            const int32_t *c = connects + (size_t)nn * e;
            int k = 0;
            while (k < nn && !mark[c[k]]) k++;
            if (k != nn) {
                again = true;
                continue;
            }
            el_color[e] = color;
            for (k = 0; k < nn; k++) mark[c[k]] = 1;
        }
        color++;
        std::fill(mark.begin(), mark.end(), 0);
    }
    return color;
}

template <class F>
static void parallel_for(int64_t n, F f)
{
    unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    if (n < 4096 || nt == 1) {
        for (int64_t i = 0; i < n; i++) f(i);
        return;
    }
    std::vector<std::thread> th;
    const int64_t chunk = (n + nt - 1) / nt;
    for (unsigned t = 0; t < nt; t++) {
        const int64_t lo = t * chunk, hi = std::min<int64_t>(n, lo + chunk);
        if (lo >= hi) break;
        th.emplace_back([=] {
            for (int64_t i = lo; i < hi; i++) f(i);
        });
    }
    for (auto &x : th) x.join();
}

// SELL-32 layout of the block pattern.  With sorted rows the warps of a
// slice run rows of one length, while every row keeps its own block order
// and stays inside the reduction block that owns it in node order.
std::string build_sell(const Setup &s, bool sorted, bool pair, SellLayout &L)
{
    L.pair = pair;
    const int64_t ns = (s.n_nodes + 31) / 32;
    std::vector<int32_t> deg(s.n_nodes);
    for (int32_t i = 0; i < s.n_nodes; i++) deg[i] = (int32_t)(s.row_ptr[i + 1] - s.row_ptr[i]);
    L.sell_node.resize(s.n_nodes);
    for (int32_t i = 0; i < s.n_nodes; i++) L.sell_node[i] = i;
    if (sorted)
        for (int64_t w0 = 0; w0 < s.n_nodes; w0 += kRedBlock) {
            const int64_t w1 = std::min<int64_t>(s.n_nodes, w0 + kRedBlock);
            std::stable_sort(L.sell_node.begin() + w0, L.sell_node.begin() + w1,
                             [&](int32_t a, int32_t b) { return deg[a] > deg[b]; });
        }
    L.rowlen.resize(s.n_nodes);
    for (int32_t t = 0; t < s.n_nodes; t++) L.rowlen[t] = deg[L.sell_node[t]];
    L.slice_base.assign((size_t)ns + 1, 0);
    for (int64_t sl = 0; sl < ns; sl++) {
        int32_t w = 0;
        for (int64_t t = sl * 32; t < std::min<int64_t>(s.n_nodes, sl * 32 + 32); t++) w = std::max(w, L.rowlen[t]);
        if (pair) w += w & 1;
        L.slice_base[sl + 1] = L.slice_base[sl] + 32 * (int64_t)w;
    }
    L.n_sell = L.slice_base[ns];
    if (L.n_sell > INT32_MAX) return "matrix too large for 32-bit block slots";
    L.sell_col.assign((size_t)L.n_sell, 0);
    L.bsr_to_sell.resize((size_t)s.n_blocks);
    L.diag_blk.resize(s.n_nodes);
    for (int32_t t = 0; t < s.n_nodes; t++) {
        const int32_t i = L.sell_node[t];
        for (int64_t j = 0; j < L.rowlen[t]; j++) {
            const int64_t slot = sell_slot(L, t, j);
            const int32_t c = s.col[s.row_ptr[i] + j];
            L.sell_col[slot] = c;
            L.bsr_to_sell[s.row_ptr[i] + j] = slot;
            if (c == i) L.diag_blk[i] = slot;
        }
        for (int64_t j = L.rowlen[t]; j < (int64_t)(L.slice_base[t / 32 + 1] - L.slice_base[t / 32]) / 32; j++)
            L.sell_col[sell_slot(L, t, j)] = i;
    }
    const int nn = s.nn, nd = s.nd;
    L.el_blk.resize((size_t)s.n_el * nn * nn);
    parallel_for(s.n_el, [&](int64_t e) {
        for (int a = 0; a < nn; a++) {
            const int32_t r = s.dofs[(size_t)e * nd + 2 * a] >> 1;
            const int32_t *b0 = s.col.data() + s.row_ptr[r], *b1 = s.col.data() + s.row_ptr[r + 1];
            for (int b = 0; b < nn; b++) {
                const int32_t c = s.dofs[(size_t)e * nd + 2 * b] >> 1;
                const int64_t j = std::lower_bound(b0, b1, c) - b0;
                L.el_blk[((size_t)e * nn + a) * nn + b] = (int32_t)L.bsr_to_sell[s.row_ptr[r] + j];
            }
        }
    });
    return "";
}

// Upper-only FP32 layout.  The FP32 tangent is symmetric block for block:
// the assembly adds each element entry and its mirror with the same value, in
// the same colour order, so the stored lower block (i, j) is exactly the
// transpose of (j, i).  Row i keeps only (i, c >= i), diagonal first, in slot
// pairs with rows in node order; an SpMV reads a lower block as the transpose
// of row j's block at position q.  Summing the lower blocks first (ascending
// j) and then the stored ones keeps the ascending-column order of the full
// layout, so every SpMV gives the same bits at half the tangent bytes.
std::string build_sell_sym(const Setup &s, SellLayout &L)
{
    L = SellLayout();
    L.pair = true;
    L.sym = true;
    const int32_t n = s.n_nodes;
    const int64_t ns = ((int64_t)n + 31) / 32;
    std::vector<int64_t> first(n);   // index of the diagonal block in row i's nodal list
    L.sell_node.resize(n);
    L.rowlen.resize(n);
    for (int32_t i = 0; i < n; i++) {
        L.sell_node[i] = i;
        const int32_t *c0 = s.col.data() + s.row_ptr[i], *c1 = s.col.data() + s.row_ptr[i + 1];
        const int32_t *d = std::lower_bound(c0, c1, i);
        if (d == c1 || *d != i) return "a row has no diagonal block";
        first[i] = d - c0;
        L.rowlen[i] = (int32_t)(c1 - d);
    }
    L.slice_base.assign((size_t)ns + 1, 0);
    for (int64_t sl = 0; sl < ns; sl++) {
        int32_t w = 0;
        for (int64_t t = sl * 32; t < std::min<int64_t>(n, sl * 32 + 32); t++) w = std::max(w, L.rowlen[t]);
        w += w & 1;
        L.slice_base[sl + 1] = L.slice_base[sl] + 32 * (int64_t)w;
    }
    L.n_sell = L.slice_base[ns];
    if (L.n_sell > INT32_MAX / 2) return "matrix too large for 32-bit block slots";
    L.sell_col.assign((size_t)L.n_sell, 0);
    L.bsr_to_sell.assign((size_t)s.n_blocks, -1);
    L.diag_blk.resize(n);
    for (int32_t i = 0; i < n; i++) {
        for (int64_t k = 0; k < L.rowlen[i]; k++) {
            const int64_t slot = sell_slot(L, i, k);
            L.sell_col[slot] = s.col[s.row_ptr[i] + first[i] + k];
            L.bsr_to_sell[s.row_ptr[i] + first[i] + k] = slot;
        }
        for (int64_t k = L.rowlen[i]; k < (L.slice_base[i / 32 + 1] - L.slice_base[i / 32]) / 32; k++)
            L.sell_col[sell_slot(L, i, k)] = i;
        L.diag_blk[i] = sell_slot(L, i, 0);
    }
    // lower blocks: -2 - slot of the stored twin; (position, stencil) lists
    std::map<std::vector<int32_t>, int> index;
    std::vector<int32_t> key;
    L.tpat_id.resize(n);
    for (int32_t i = 0; i < n; i++) {
        key.clear();
        for (int64_t k = 0; k < first[i]; k++) {
            const int32_t j = s.col[s.row_ptr[i] + k];
            const int32_t *c0 = s.col.data() + s.row_ptr[j] + first[j], *c1 = s.col.data() + s.row_ptr[j + 1];
            const int32_t *f = std::lower_bound(c0, c1, i);
            if (f == c1 || *f != i) return "the block pattern is not symmetric";
            const int32_t q = (int32_t)(f - c0);
            L.bsr_to_sell[s.row_ptr[i] + k] = -2 - sell_slot(L, j, q);
            key.push_back(j - i);
            key.push_back(q);
        }
        if ((int)key.size() > 2 * kPatLen) return "a row has more lower blocks than a stencil holds";
        auto it = index.find(key);
        if (it == index.end()) {
            if ((int)index.size() == kPatMax) return "more transposed stencils than 8-bit ids";
            it = index.emplace(key, (int)index.size()).first;
            L.tpat.resize((size_t)index.size() * kPatLen * 2, 0);
            L.tpat_len.push_back((int32_t)key.size() / 2);
            std::copy(key.begin(), key.end(), L.tpat.begin() + (size_t)it->second * kPatLen * 2);
        }
        L.tpat_id[i] = (uint8_t)it->second;
    }
    L.n_tpat = (int)index.size();
    const int nn = s.nn, nd = s.nd;
    L.el_blk.resize((size_t)s.n_el * nn * nn);
    parallel_for(s.n_el, [&](int64_t e) {
        for (int a = 0; a < nn; a++) {
            const int32_t r = s.dofs[(size_t)e * nd + 2 * a] >> 1;
            const int32_t *b0 = s.col.data() + s.row_ptr[r], *b1 = s.col.data() + s.row_ptr[r + 1];
            for (int b = 0; b < nn; b++) {
                const int32_t c = s.dofs[(size_t)e * nd + 2 * b] >> 1;
                const int64_t j = std::lower_bound(b0, b1, c) - b0;
                const int64_t slot = L.bsr_to_sell[s.row_ptr[r] + j];
                L.el_blk[((size_t)e * nn + a) * nn + b] = c >= r ? (int32_t)slot : -1;
            }
        }
    });
    build_row_stencils(L);
    if (L.n_pat == 0) return "the upper lists have no row stencils";
    return "";
}

// Row stencils: the column offsets (column - node) of a row in slot order.
// On a structured node grid a few dozen distinct stencils cover every row
// (interior vertex, edge and centre nodes of the quadrilaterals plus their
// boundary variants), so an SpMV can form a row's columns from its node and
// an 8-bit stencil id instead of loading one index per block.  With a row
// longer than kPatLen or more than kPatMax stencils (unstructured numbering)
// the layout keeps only its explicit columns (n_pat = 0).
void build_row_stencils(SellLayout &L)
{
    L.n_pat = 0;
    L.pat_id.clear();
    L.pat_off.clear();
    const int32_t n = (int32_t)L.rowlen.size();
    std::map<std::vector<int32_t>, int> index;
    std::vector<uint8_t> id((size_t)n);
    std::vector<int32_t> off, key;
    for (int32_t t = 0; t < n; t++) {
        const int32_t i = L.sell_node[t];
        const int len = L.rowlen[t];
        if (len > kPatLen) return;
        key.resize((size_t)len);
        for (int k = 0; k < len; k++) key[k] = L.sell_col[(size_t)sell_slot(L, t, k)] - i;
        // rows of a grid line repeat the stencils of the rows two and four before
        int p = -1;
        for (int back = 2; back <= 4 && p < 0; back += 2) {
            if (t < back || L.rowlen[t - back] != len) continue;
            const int q = id[(size_t)(t - back)];
            if (std::equal(key.begin(), key.end(), off.begin() + (size_t)q * kPatLen)) p = q;
        }
        if (p < 0) {
            auto it = index.find(key);
            if (it != index.end()) {
                p = it->second;
            } else {
                if ((int)index.size() == kPatMax) return;
                p = (int)index.size();
                index.emplace(key, p);
                off.resize((size_t)(p + 1) * kPatLen, 0);
                std::copy(key.begin(), key.end(), off.begin() + (size_t)p * kPatLen);
            }
        }
        id[(size_t)t] = (uint8_t)p;
    }
    L.pat_id = std::move(id);
    L.pat_off = std::move(off);
    L.n_pat = (int)index.size();
}

std::string build_setup(const ipfem_mesh *m, const ipfem_material *mat, Setup &s)
{
    if (!m || !mat) return "null mesh or material";
    if (m->n_elements <= 0 || m->n_nodes <= 0) return "empty mesh";
    if (!m->connects || !m->weight || (!m->dphi && !m->block_storage)) return "mesh arrays missing";
    if ((int64_t)m->n_nodes * 2 > INT32_MAX) return "too many nodes";
    if (m->order < 0 || m->order > IPFEM_MAX_ORDER) return "element order must be 1, 2 or 3";
    s.order = m->order == 0 ? 2 : m->order;
    s.nn = s.nq = (s.order + 1) * (s.order + 1);
    s.nd = 2 * s.nn;
    const int nn = s.nn, nq = s.nq, nd = s.nd;
    s.n_el = m->n_elements;
    s.n_nodes = m->n_nodes;
    s.neq = 2 * m->n_nodes;
    s.n_ip = (int64_t)s.n_el * nq;
    for (int64_t k = 0; k < (int64_t)s.n_el * nn; k++)
        if (m->connects[k] < 0 || m->connects[k] >= s.n_nodes) return "connect index out of range";
    for (int32_t e = 0; e < s.n_el; e++) {
        const int32_t *c = m->connects + (size_t)nn * e;
        for (int a = 0; a < nn; a++)
            for (int b = a + 1; b < nn; b++)
                if (c[a] == c[b]) return "repeated connect in an element";
    }
    // element blocks
    s.dphi.resize((size_t)s.n_el * nq * 2 * nn);
    if (m->dphi) {
        std::memcpy(s.dphi.data(), m->dphi, s.dphi.size() * sizeof(double));
    } else {
        // fStorage (3*npts) x (2*nshape) row-major: row 3q+comp+jdim, column 2n+comp
        // (TPZNumericalIntegrator.cpp:371-381)
        for (int32_t e = 0; e < s.n_el; e++) {
            const double *B = m->block_storage + (size_t)e * 3 * nq * nd;
            for (int q = 0; q < nq; q++)
                for (int n = 0; n < nn; n++) {
                    const double dx = B[(3 * q + 0) * nd + 2 * n], dy = B[(3 * q + 1) * nd + 2 * n];
                    if (B[(3 * q + 1) * nd + 2 * n + 1] != dx || B[(3 * q + 2) * nd + 2 * n + 1] != dy ||
                        B[(3 * q + 0) * nd + 2 * n + 1] != 0.0 || B[(3 * q + 2) * nd + 2 * n] != 0.0)
                        return "block_storage is not a 2-D strain block (element " + std::to_string(e) + ")";
                    s.dphi[((size_t)e * nq + q) * 2 * nn + n] = dx;
                    s.dphi[((size_t)e * nq + q) * 2 * nn + nn + n] = dy;
                }
        }
    }
    s.weight.assign(m->weight, m->weight + s.n_ip);
    // dof map (TPZNumericalIntegrator.cpp:429-443): connect sequence x 2
    s.dofs.resize((size_t)s.n_el * nd);
    for (size_t k = 0; k < (size_t)s.n_el * nn; k++) {
        s.dofs[2 * k] = 2 * m->connects[k];
        s.dofs[2 * k + 1] = 2 * m->connects[k] + 1;
    }
    // colouring
    s.el_color.resize(s.n_el);
    s.n_colors = greedy_coloring_nn(s.n_el, s.n_nodes, nn, m->connects, s.el_color.data());
    if (s.n_colors > kMaxColors) return "more than 16 colours";
    s.color_ptr.assign(s.n_colors + 1, 0);
    for (int32_t e = 0; e < s.n_el; e++) s.color_ptr[s.el_color[e] + 1]++;
    for (int c = 0; c < s.n_colors; c++) s.color_ptr[c + 1] += s.color_ptr[c];
    s.color_els.resize(s.n_el);
    {
        std::vector<int32_t> fill(s.n_colors, 0);
        for (int32_t e = 0; e < s.n_el; e++) {
            const int c = s.el_color[e];
            s.color_els[s.color_ptr[c] + fill[c]++] = e;
        }
    }
    s.inc.assign((size_t)s.n_colors * s.n_nodes, -1);
    for (int32_t e = 0; e < s.n_el; e++)
        for (int ln = 0; ln < nn; ln++)
            s.inc[(size_t)s.el_color[e] * s.n_nodes + m->connects[(size_t)nn * e + ln]] = e * nn + ln;
    // nodal block pattern
    {
        std::vector<int64_t> cap((size_t)s.n_nodes + 1, 0);
        for (size_t k = 0; k < (size_t)s.n_el * nn; k++) cap[m->connects[k] + 1] += nn;
        for (int32_t i = 0; i < s.n_nodes; i++) cap[i + 1] += cap[i];
        std::vector<int32_t> tmp((size_t)cap[s.n_nodes]);
        std::vector<int32_t> deg((size_t)s.n_nodes, 0);
        for (int32_t e = 0; e < s.n_el; e++)
            for (int a = 0; a < nn; a++) {
                const int32_t r = m->connects[(size_t)nn * e + a];
                for (int b = 0; b < nn; b++) tmp[cap[r] + deg[r]++] = m->connects[(size_t)nn * e + b];
            }
        s.row_ptr.assign((size_t)s.n_nodes + 1, 0);
        parallel_for(s.n_nodes, [&](int64_t i) {
            int32_t *b = tmp.data() + cap[i];
            std::sort(b, b + deg[i]);
            deg[i] = (int32_t)(std::unique(b, b + deg[i]) - b);
        });
        for (int32_t i = 0; i < s.n_nodes; i++) s.row_ptr[i + 1] = s.row_ptr[i] + deg[i];
        s.n_blocks = s.row_ptr[s.n_nodes];
        s.col.resize((size_t)s.n_blocks);
        for (int32_t i = 0; i < s.n_nodes; i++)
            std::memcpy(s.col.data() + s.row_ptr[i], tmp.data() + cap[i], (size_t)deg[i] * sizeof(int32_t));
    }
    {
        const std::string e = build_sell(s, true, false, s.sell);
        if (!e.empty()) return e;
        build_row_stencils(s.sell);
    }
    // boundary conditions and loads
    s.fixed.assign((size_t)s.neq, 0);
    if (m->fixed) std::memcpy(s.fixed.data(), m->fixed, (size_t)s.neq);
    s.f0.assign((size_t)s.neq, 0.0);
    s.df.assign((size_t)s.neq, 0.0);
    if (m->f0) std::memcpy(s.f0.data(), m->f0, (size_t)s.neq * sizeof(double));
    if (m->df) std::memcpy(s.df.data(), m->df, (size_t)s.neq * sizeof(double));
    // material
    if (!(mat->E > 0) || !(mat->nu > -1.0 && mat->nu < 0.5)) return "invalid elastic constants";
    elastic_constants(mat->E, mat->nu, s.el);
    s.mat.resize((size_t)5 * s.n_el);
    for (int32_t e = 0; e < s.n_el; e++) {
        const double c = mat->el_cohesion ? mat->el_cohesion[e] : mat->cohesion;
        const double phi = mat->el_phi ? mat->el_phi[e] : mat->phi;
        const double psi = mat->el_phi ? phi : mat->psi;
        s.mat[e] = c;
        s.mat[(size_t)s.n_el + e] = std::sin(phi);
        s.mat[2 * (size_t)s.n_el + e] = std::cos(phi);
        s.mat[3 * (size_t)s.n_el + e] = std::tan(phi);
        s.mat[4 * (size_t)s.n_el + e] = std::sin(psi);
    }
    // in-situ seed: eps_p0 = -C^{-1} sigma0 (ComputeStrain, FunctionsStressStrain.h:73-81)
    for (int k = 0; k < 4; k++) s.sigma0[k] = mat->sigma0[k];
    {
        const double sxx = mat->sigma0[0], sxy = mat->sigma0[1], syy = mat->sigma0[2], szz = mat->sigma0[3];
        const double exx = s.el.c1 * sxx - s.el.c2 * (syy + szz);
        const double eyy = s.el.c1 * syy - s.el.c2 * (sxx + szz);
        const double ezz = s.el.c1 * szz - s.el.c2 * (syy + sxx);
        const double exy = s.el.inv_mu * sxy;
        s.eps_p0[0] = -exx;
        s.eps_p0[1] = -exy;
        s.eps_p0[2] = -eyy;
        s.eps_p0[3] = -ezz;
    }
    return "";
}

// ------------------------------------------------------ wellbore provider

static uint64_t sm64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}

static double urand(uint64_t seed, uint64_t e, uint64_t k)
{
    return (double)(sm64(seed * 0x100000001B3ULL + 4 * e + k) >> 11) * 0x1.0p-53;
}

static const int kRefA[9] = {-1, 1, 1, -1, 0, 1, 0, -1, 0};
static const int kRefB[9] = {-1, -1, 1, 1, -1, 0, 1, 0, 0};

// order-2 Lagrange functions on -1, 0, 1 (closed forms)
static double lag(int a, double x)
{
    if (a < 0) return 0.5 * x * (x - 1.0);
    if (a == 0) return 1.0 - x * x;
    return 0.5 * x * (x + 1.0);
}

static double dlag(int a, double x)
{
    if (a < 0) return x - 0.5;
    if (a == 0) return -2.0 * x;
    return x + 0.5;
}

// 1-D Lagrange function a of order p on the equispaced nodes t_m = -1 + 2m/p
// and its derivative (orders 1 and 3)
static double lagp(int p, int a, double x)
{
    const double ta = -1.0 + 2.0 * a / p;
    double num = 1.0, den = 1.0;
    for (int m = 0; m <= p; m++) {
        if (m == a) continue;
        const double tm = -1.0 + 2.0 * m / p;
        num = num * (x - tm);
        den = den * (ta - tm);
    }
    return num / den;
}

static double dlagp(int p, int a, double x)
{
    const double ta = -1.0 + 2.0 * a / p;
    double s = 0.0;
    for (int k = 0; k <= p; k++) {
        if (k == a) continue;
        const double tk = -1.0 + 2.0 * k / p;
        double prod = 1.0 / (ta - tk);
        for (int m = 0; m <= p; m++) {
            if (m == a || m == k) continue;
            const double tm = -1.0 + 2.0 * m / p;
            prod = prod * ((x - tm) / (ta - tm));
        }
        s = s + prod;
    }
    return s;
}

// index-space position (a, b) in [0, p]^2 of connect n of an order-p element:
// vertices, the p-1 nodes of each edge in traversal order, interior row by row
static void ref_node(int p, int n, int &a, int &b)
{
    const int vx[4] = {0, p, p, 0}, vy[4] = {0, 0, p, p};
    if (n < 4) {
        a = vx[n];
        b = vy[n];
        return;
    }
    n -= 4;
    if (n < 4 * (p - 1)) {
        const int e = n / (p - 1), k = n % (p - 1) + 1;
        if (e == 0) { a = k; b = 0; }
        else if (e == 1) { a = p; b = k; }
        else if (e == 2) { a = p - k; b = p; }
        else { a = 0; b = p - k; }
        return;
    }
    n -= 4 * (p - 1);
    a = n % (p - 1) + 1;
    b = n / (p - 1) + 1;
}

// Gauss points and weights, p + 1 per direction
static void gauss(int p, double *gp, double *gw)
{
    if (p == 1) {
        const double g = 1.0 / std::sqrt(3.0);
        gp[0] = -g; gp[1] = g;
        gw[0] = 1.0; gw[1] = 1.0;
    } else if (p == 2) {
        const double g = std::sqrt(0.6);
        gp[0] = -g; gp[1] = 0.0; gp[2] = g;
        gw[0] = 5.0 / 9.0; gw[1] = 8.0 / 9.0; gw[2] = 5.0 / 9.0;
    } else {
        const double a = std::sqrt(3.0 / 7.0 - 2.0 / 7.0 * std::sqrt(6.0 / 5.0));
        const double b = std::sqrt(3.0 / 7.0 + 2.0 / 7.0 * std::sqrt(6.0 / 5.0));
        const double wa = (18.0 + std::sqrt(30.0)) / 36.0, wb = (18.0 - std::sqrt(30.0)) / 36.0;
        gp[0] = -b; gp[1] = -a; gp[2] = a; gp[3] = b;
        gw[0] = wb; gw[1] = wa; gw[2] = wa; gw[3] = wb;
    }
}

// d(phi)/dx, d(phi)/dy and w|detJ| of a bilinear-geometry element of order p
// at its Gauss points (point q = (p+1)*i_eta + i_xi); shape functions are the
// tensor-product Lagrange functions of its connects
static void element_dphi(int p, const double *X, const double *Y, double *dphi, double *w)
{
    const int n1 = p + 1, nn = n1 * n1, nq = n1 * n1;
    double gp[4], gw[4];
    gauss(p, gp, gw);
    for (int iq = 0; iq < nq; iq++) {
        const int ix = iq % n1, iy = iq / n1;
        const double xi = gp[ix], eta = gp[iy];
        const double dpx[4] = {-(1.0 - eta) / 4.0, (1.0 - eta) / 4.0, (1.0 + eta) / 4.0, -(1.0 + eta) / 4.0};
        const double dpe[4] = {-(1.0 - xi) / 4.0, -(1.0 + xi) / 4.0, (1.0 + xi) / 4.0, (1.0 - xi) / 4.0};
        double x_xi = dpx[0] * X[0], x_eta = dpe[0] * X[0];
        double y_xi = dpx[0] * Y[0], y_eta = dpe[0] * Y[0];
        for (int v = 1; v < 4; v++) {
            x_xi = x_xi + dpx[v] * X[v];
            x_eta = x_eta + dpe[v] * X[v];
            y_xi = y_xi + dpx[v] * Y[v];
            y_eta = y_eta + dpe[v] * Y[v];
        }
        const double det = x_xi * y_eta - x_eta * y_xi;
        const double xi_x = y_eta / det, xi_y = -x_eta / det;
        const double eta_x = -y_xi / det, eta_y = x_xi / det;
        w[iq] = (gw[ix] * gw[iy]) * std::fabs(det);
        for (int n = 0; n < nn; n++) {
            double Nxi, Neta;
            if (p == 2) {
                Nxi = dlag(kRefA[n], xi) * lag(kRefB[n], eta);
                Neta = lag(kRefA[n], xi) * dlag(kRefB[n], eta);
            } else {
                int a, b;
                ref_node(p, n, a, b);
                Nxi = dlagp(p, a, xi) * lagp(p, b, eta);
                Neta = lagp(p, a, xi) * dlagp(p, b, eta);
            }
            dphi[iq * 2 * nn + n] = Nxi * xi_x + Neta * eta_x;
            dphi[iq * 2 * nn + nn + n] = Nxi * xi_y + Neta * eta_y;
        }
    }
}

// barycentric index (i, j, k), i + j + k = p, of connect n of an order-p
// triangle: vertices, the p-1 nodes of each edge in traversal order (edges
// v0v1, v1v2, v2v0), the interior node (p = 3)
static void tri_node(int p, int n, int &i, int &j, int &k)
{
    if (n < 3) {
        i = n == 0 ? p : 0;
        j = n == 1 ? p : 0;
        k = n == 2 ? p : 0;
        return;
    }
    n -= 3;
    if (n < 3 * (p - 1)) {
        const int e = n / (p - 1), m = n % (p - 1) + 1;
        if (e == 0) { i = p - m; j = m; k = 0; }
        else if (e == 1) { i = 0; j = p - m; k = m; }
        else { i = m; j = 0; k = p - m; }
        return;
    }
    i = j = k = 1;
}

// l_m(L) = prod_{s<m} (p L - s)/(s + 1) and its derivative in L
static void bary_factor(int p, int m, double L, double &v, double &d)
{
    v = 1.0;
    d = 0.0;
    for (int s = 0; s < m; s++) {
        const double f = (p * L - s) / (s + 1), df = (double)p / (s + 1);
        d = d * f + v * df;
        v = v * f;
    }
}

// An order-p triangle (Lagrange functions on the equispaced barycentric
// lattice, affine geometry from its 3 vertex connects) in the block shape of
// the order-p quadrilateral: its (p+1)(p+2)/2 connects fill the first
// columns, the remaining columns (ghost connects) are zero; the (p+1)^2
// points are the collapsed Gauss rule xi = u, eta = v (1 - u) on the unit
// triangle (u, v on the Gauss points of [0, 1]), weight w_u w_v (1 - u)|det|,
// exact for the degree-2p integrands of the tangent.
void tri_element_dphi(int p, const double *X, const double *Y, double *dphi, double *w)
{
    const int n1 = p + 1, nn = n1 * n1, nq = n1 * n1, nt = (p + 1) * (p + 2) / 2;
    double gp[4], gw[4];
    gauss(p, gp, gw);
    const double x1 = X[1] - X[0], x2 = X[2] - X[0], y1 = Y[1] - Y[0], y2 = Y[2] - Y[0];
    const double det = x1 * y2 - x2 * y1;
    const double xi_x = y2 / det, xi_y = -x2 / det, eta_x = -y1 / det, eta_y = x1 / det;
    for (int t = 0; t < nq * 2 * nn; t++) dphi[t] = 0.0;
    for (int iq = 0; iq < nq; iq++) {
        const int iu = iq % n1, iv = iq / n1;
        const double u = 0.5 * (1.0 + gp[iu]), v = 0.5 * (1.0 + gp[iv]);
        const double xi = u, eta = v * (1.0 - u);
        w[iq] = ((0.5 * gw[iu]) * (0.5 * gw[iv])) * (1.0 - u) * std::fabs(det);
        const double L[3] = {1.0 - xi - eta, xi, eta};
        for (int n = 0; n < nt; n++) {
            int b[3];
            tri_node(p, n, b[0], b[1], b[2]);
            double f[3], df[3];
            for (int c = 0; c < 3; c++) bary_factor(p, b[c], L[c], f[c], df[c]);
            const double dL0 = df[0] * f[1] * f[2], dL1 = f[0] * df[1] * f[2], dL2 = f[0] * f[1] * df[2];
            const double Nxi = dL1 - dL0, Neta = dL2 - dL0;
            dphi[iq * 2 * nn + n] = Nxi * xi_x + Neta * eta_x;
            dphi[iq * 2 * nn + nn + n] = Nxi * xi_y + Neta * eta_y;
        }
    }
}

void element_blocks_dphi(int order, int64_t n_el, const int32_t *connects, const double *node_xy, double *dphi,
                         double *weight, const uint8_t *shape)
{
    const int nn = (order + 1) * (order + 1), nq = nn;
    parallel_for(n_el, [&](int64_t e) {
        double X[4], Y[4];
        const int nv = (shape && shape[e]) ? 3 : 4;
        for (int v = 0; v < nv; v++) {
            X[v] = node_xy[2 * (size_t)connects[(size_t)nn * e + v]];
            Y[v] = node_xy[2 * (size_t)connects[(size_t)nn * e + v] + 1];
        }
        if (nv == 3) tri_element_dphi(order, X, Y, dphi + e * nq * 2 * nn, weight + e * nq);
        else element_dphi(order, X, Y, dphi + e * nq * 2 * nn, weight + e * nq);
    });
}

static void seg_load(const double *xy, int32_t P, int32_t M, int32_t Q, int sgn, double sxx, double sxy, double syy,
                     double *f)
{
    const double dx = xy[2 * (size_t)Q] - xy[2 * (size_t)P];
    const double dy = xy[2 * (size_t)Q + 1] - xy[2 * (size_t)P + 1];
    const double L = std::sqrt(dx * dx + dy * dy);
    const double nx = sgn > 0 ? dy / L : -dy / L;
    const double ny = sgn > 0 ? -dx / L : dx / L;
    const double tx = sxx * nx + sxy * ny;
    const double ty = sxy * nx + syy * ny;
    const double we = L / 6.0, wm = 2.0 * L / 3.0;
    f[2 * (size_t)P] += tx * we;
    f[2 * (size_t)P + 1] += ty * we;
    f[2 * (size_t)M] += tx * wm;
    f[2 * (size_t)M + 1] += ty * wm;
    f[2 * (size_t)Q] += tx * we;
    f[2 * (size_t)Q + 1] += ty * we;
}

}  // namespace ipfem

using namespace ipfem;

extern "C" int32_t ipfem_color_elements_nn(int32_t n_el, int32_t n_nodes, int32_t nn, const int32_t *connects,
                                           int32_t *el_color)
{
    if (n_el <= 0 || n_nodes <= 0 || nn < 4 || !connects || !el_color) return -1;
    for (int64_t k = 0; k < (int64_t)n_el * nn; k++)
        if (connects[k] < 0 || connects[k] >= n_nodes) return -1;
    return greedy_coloring_nn(n_el, n_nodes, nn, connects, el_color);
}

extern "C" int32_t ipfem_color_elements(int32_t n_el, int32_t n_nodes, const int32_t *connects, int32_t *el_color)
{
    return ipfem_color_elements_nn(n_el, n_nodes, 9, connects, el_color);
}

extern "C" void ipfem_wellbore_default(ipfem_wellbore_params *p, int32_t n)
{
    std::memset(p, 0, sizeof *p);
    p->nr = n;
    p->nt = n;
    p->r_in = 0.1;
    p->r_out = 4.0;
    p->grading = std::pow(1.05, 40.0 / (double)n);
    p->E = 15000.0;
    p->nu = 0.2;
    p->cohesion = 10.0;
    p->phi_deg = 30.0;
    p->psi_deg = 30.0;
    p->sxx0 = -40.0;
    p->syy0 = -50.0;
    p->sxy0 = 0.0;
    p->szz0 = 0.2 * (-40.0 + -50.0);
    p->pw_final = -10.0;
    p->material_mode = 0;
    p->c_cv = 0.2;
    p->phi_lo_deg = 25.0;
    p->phi_hi_deg = 35.0;
    p->seed = 20260101ULL;
}

extern "C" void ipfem_wellbore_free(ipfem_wellbore *w)
{
    if (!w) return;
    std::free(w->node_xy);
    std::free(w->connects);
    std::free(w->dphi);
    std::free(w->weight);
    std::free(w->f0);
    std::free(w->df);
    std::free(w->el_cohesion);
    std::free(w->el_phi);
    std::free(w->fixed);
    std::free(w->el_shape);
    delete w;
}

extern "C" ipfem_status ipfem_wellbore_build(const ipfem_wellbore_params *prm, ipfem_wellbore **out)
{
    if (!prm || !out) return IPFEM_INVALID;
    *out = nullptr;
    const int nr = prm->nr, nt = prm->nt;
    if (nr < 1 || nt < 1 || !(prm->r_out > prm->r_in) || !(prm->r_in > 0) || !(prm->grading > 0))
        return IPFEM_INVALID;
    const int gr = 2 * nr + 1, gt = 2 * nt + 1;
    const int64_t n_el = (int64_t)nr * nt, n_nodes = (int64_t)gr * gt;
    if (n_nodes * 2 > INT32_MAX || n_el * 81 > INT32_MAX) return IPFEM_INVALID;
    ipfem_wellbore *w = new (std::nothrow) ipfem_wellbore();
    if (!w) return IPFEM_OOM;
    std::memset(w, 0, sizeof *w);
    const int64_t neq = 2 * n_nodes;
    w->node_xy = (double *)std::calloc((size_t)n_nodes * 2, sizeof(double));
    w->connects = (int32_t *)std::calloc((size_t)n_el * 9, sizeof(int32_t));
    w->dphi = (double *)std::calloc((size_t)n_el * 162, sizeof(double));
    w->weight = (double *)std::calloc((size_t)n_el * 9, sizeof(double));
    w->f0 = (double *)std::calloc((size_t)neq, sizeof(double));
    w->df = (double *)std::calloc((size_t)neq, sizeof(double));
    w->fixed = (uint8_t *)std::calloc((size_t)neq, 1);
    if (!w->node_xy || !w->connects || !w->dphi || !w->weight || !w->f0 || !w->df || !w->fixed) {
        ipfem_wellbore_free(w);
        return IPFEM_OOM;
    }
    // vertex radii (geometric grading) and angles
    std::vector<double> r((size_t)nr + 1), vxy((size_t)(nr + 1) * (nt + 1) * 2);
    const double q = prm->grading;
    const double h0 = (q == 1.0) ? (prm->r_out - prm->r_in) / (double)nr
                                 : (prm->r_out - prm->r_in) * (q - 1.0) / (std::pow(q, (double)nr) - 1.0);
    r[0] = prm->r_in;
    for (int i = 0; i < nr - 1; i++) r[i + 1] = r[i] + h0 * std::pow(q, (double)i);
    r[nr] = prm->r_out;
    const double dth = (0.5 * M_PI) / (double)nt;
    for (int j = 0; j <= nt; j++) {
        const double th = (double)j * dth;
        const double c = std::cos(th), sn = std::sin(th);
        for (int i = 0; i <= nr; i++) {
            double *v = &vxy[2 * ((size_t)j * (nr + 1) + i)];
            if (j == 0) { v[0] = r[i]; v[1] = 0.0; }
            else if (j == nt) { v[0] = 0.0; v[1] = r[i]; }
            else { v[0] = r[i] * c; v[1] = r[i] * sn; }
        }
    }
    for (int b = 0; b < gt; b++)
        for (int a = 0; a < gr; a++) {
            double *o = &w->node_xy[2 * ((size_t)b * gr + a)];
            const int i0 = a / 2, j0 = b / 2, i1 = (a + 1) / 2, j1 = (b + 1) / 2;
            const double *v00 = &vxy[2 * ((size_t)j0 * (nr + 1) + i0)];
            const double *v10 = &vxy[2 * ((size_t)j0 * (nr + 1) + i1)];
            const double *v11 = &vxy[2 * ((size_t)j1 * (nr + 1) + i1)];
            const double *v01 = &vxy[2 * ((size_t)j1 * (nr + 1) + i0)];
            if (!(a & 1) && !(b & 1)) { o[0] = v00[0]; o[1] = v00[1]; }
            else if ((a & 1) && !(b & 1)) { o[0] = 0.5 * (v00[0] + v10[0]); o[1] = 0.5 * (v00[1] + v10[1]); }
            else if (!(a & 1) && (b & 1)) { o[0] = 0.5 * (v00[0] + v01[0]); o[1] = 0.5 * (v00[1] + v01[1]); }
            else {
                o[0] = 0.25 * (((v00[0] + v10[0]) + v11[0]) + v01[0]);
                o[1] = 0.25 * (((v00[1] + v10[1]) + v11[1]) + v01[1]);
            }
        }
    auto nid = [gr](int a, int b) { return (int32_t)(b * gr + a); };
    for (int j = 0; j < nt; j++)
        for (int i = 0; i < nr; i++) {
            int32_t *c = &w->connects[9 * ((size_t)j * nr + i)];
            const int a0 = 2 * i, b0 = 2 * j;
            c[0] = nid(a0, b0); c[1] = nid(a0 + 2, b0); c[2] = nid(a0 + 2, b0 + 2); c[3] = nid(a0, b0 + 2);
            c[4] = nid(a0 + 1, b0); c[5] = nid(a0 + 2, b0 + 1); c[6] = nid(a0 + 1, b0 + 2); c[7] = nid(a0, b0 + 1);
            c[8] = nid(a0 + 1, b0 + 1);
        }
    element_blocks_dphi(2, n_el, w->connects, w->node_xy, w->dphi, w->weight);
    for (int a = 0; a < gr; a++) {
        w->fixed[2 * (size_t)nid(a, 0) + 1] = 1;
        w->fixed[2 * (size_t)nid(a, gt - 1) + 0] = 1;
    }
    {
        std::vector<double> fo((size_t)neq, 0.0), fw0((size_t)neq, 0.0), fw1((size_t)neq, 0.0);
        for (int j = 0; j < nt; j++) {
            seg_load(w->node_xy, nid(gr - 1, 2 * j), nid(gr - 1, 2 * j + 1), nid(gr - 1, 2 * j + 2), +1, prm->sxx0,
                     prm->sxy0, prm->syy0, fo.data());
            seg_load(w->node_xy, nid(0, 2 * j), nid(0, 2 * j + 1), nid(0, 2 * j + 2), -1, prm->sxx0, prm->sxy0,
                     prm->syy0, fw0.data());
            seg_load(w->node_xy, nid(0, 2 * j), nid(0, 2 * j + 1), nid(0, 2 * j + 2), -1, prm->pw_final, 0.0,
                     prm->pw_final, fw1.data());
        }
        for (int64_t i = 0; i < neq; i++) {
            w->f0[i] = fo[i] + fw0[i];
            w->df[i] = fw1[i] - fw0[i];
        }
    }
    const double d2r = M_PI / 180.0;
    w->material.E = prm->E;
    w->material.nu = prm->nu;
    w->material.cohesion = prm->cohesion;
    w->material.phi = prm->phi_deg * d2r;
    w->material.psi = prm->psi_deg * d2r;
    w->material.sigma0[0] = prm->sxx0;
    w->material.sigma0[1] = prm->sxy0;
    w->material.sigma0[2] = prm->syy0;
    w->material.sigma0[3] = prm->szz0;
    if (prm->material_mode >= 1) {
        w->el_cohesion = (double *)std::calloc((size_t)n_el, sizeof(double));
        if (!w->el_cohesion) {
            ipfem_wellbore_free(w);
            return IPFEM_OOM;
        }
        const double s2 = std::log(1.0 + prm->c_cv * prm->c_cv);
        const double mln = std::log(prm->cohesion) - 0.5 * s2;
        const double sln = std::sqrt(s2);
        parallel_for(n_el, [&](int64_t e) {
            const double u1 = 1.0 - urand(prm->seed, (uint64_t)e, 0);
            const double u2 = urand(prm->seed, (uint64_t)e, 1);
            const double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
            w->el_cohesion[e] = std::exp(mln + sln * z);
        });
        w->material.el_cohesion = w->el_cohesion;
    }
    if (prm->material_mode >= 2) {
        w->el_phi = (double *)std::calloc((size_t)n_el, sizeof(double));
        if (!w->el_phi) {
            ipfem_wellbore_free(w);
            return IPFEM_OOM;
        }
        parallel_for(n_el, [&](int64_t e) {
            const double phi = prm->phi_lo_deg + (prm->phi_hi_deg - prm->phi_lo_deg) * urand(prm->seed, (uint64_t)e, 2);
            w->el_phi[e] = phi * d2r;
        });
        w->material.el_phi = w->el_phi;
    }
    w->mesh.n_elements = (int32_t)n_el;
    w->mesh.n_nodes = (int32_t)n_nodes;
    w->mesh.connects = w->connects;
    w->mesh.dphi = w->dphi;
    w->mesh.block_storage = nullptr;
    w->mesh.weight = w->weight;
    w->mesh.fixed = w->fixed;
    w->mesh.f0 = w->f0;
    w->mesh.df = w->df;
    w->mesh.order = 2;
    *out = w;
    return IPFEM_OK;
}
