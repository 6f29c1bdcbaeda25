// Gmsh meshes on the host: the reader that stands in for NeoPZ's
// TPZGmshReader (ReadGeometry, main.cpp:447-464; the reference's meshes are
// gmsh/wellbore_*.msh, Gmsh 4.1 ASCII), and the problem of order 1, 2 or 3
// built on them as CmeshElastoplasticity does (main.cpp:546-601): the
// elastoplastic domain on the quadrilaterals and the TBCData boundary
// conditions (main.cpp:374-446) on the tagged lines and points.
//
// Compiled with -ffp-contract=off: coordinates, element blocks and loads are
// the separately rounded results of the written expressions on every host.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "ipfem_internal.h"

using namespace ipfem;

namespace {

// whitespace tokenizer over the whole file
struct Tokens {
    std::string buf;
    size_t pos = 0;
    bool bad = false;

    void skip_ws()
    {
        while (pos < buf.size() && (buf[pos] == ' ' || buf[pos] == '\t' || buf[pos] == '\r' || buf[pos] == '\n'))
            pos++;
    }
    std::string word()
    {
        skip_ws();
        const size_t b = pos;
        while (pos < buf.size() && !(buf[pos] == ' ' || buf[pos] == '\t' || buf[pos] == '\r' || buf[pos] == '\n'))
            pos++;
        if (b == pos) bad = true;
        return buf.substr(b, pos - b);
    }
    // rest of the current line (after the last token read), without the newline
    std::string rest_of_line()
    {
        const size_t b = pos;
        while (pos < buf.size() && buf[pos] != '\n') pos++;
        std::string s = buf.substr(b, pos - b);
        if (pos < buf.size()) pos++;
        while (!s.empty() && (s.back() == '\r' || s.back() == ' ')) s.pop_back();
        return s;
    }
    long long integer()
    {
        const std::string w = word();
        char *end = nullptr;
        const long long v = std::strtoll(w.c_str(), &end, 10);
        if (w.empty() || *end) bad = true;
        return v;
    }
    double real()
    {
        const std::string w = word();
        char *end = nullptr;
        const double v = std::strtod(w.c_str(), &end);
        if (w.empty() || *end) bad = true;
        return v;
    }
};

ipfem_status gmsh_fail(const std::string &msg)
{
    set_thread_error("Gmsh: " + msg);
    return IPFEM_INVALID;
}

int32_t *dup_i32(const std::vector<int32_t> &v)
{
    int32_t *p = (int32_t *)std::malloc((v.size() ? v.size() : 1) * sizeof(int32_t));
    if (p && !v.empty()) std::memcpy(p, v.data(), v.size() * sizeof(int32_t));
    return p;
}

uint64_t edge_key(int32_t a, int32_t b)
{
    const uint32_t lo = (uint32_t)(a < b ? a : b), hi = (uint32_t)(a < b ? b : a);
    return ((uint64_t)lo << 32) | hi;
}

// consistent load of a constant traction (tx, ty) on a straight 3-connect
// edge A-M-B: the Q2 trace functions integrate to L/6, 2L/3, L/6
void edge_load(const double *xy, int32_t A, int32_t M, int32_t B, double tx, double ty, double *f)
{
    const double dx = xy[2 * (size_t)B] - xy[2 * (size_t)A];
    const double dy = xy[2 * (size_t)B + 1] - xy[2 * (size_t)A + 1];
    const double L = std::sqrt(dx * dx + dy * dy);
    const double we = L / 6.0, wm = 2.0 * L / 3.0;
    f[2 * (size_t)A] += tx * we;
    f[2 * (size_t)A + 1] += ty * we;
    f[2 * (size_t)M] += tx * wm;
    f[2 * (size_t)M + 1] += ty * wm;
    f[2 * (size_t)B] += tx * we;
    f[2 * (size_t)B + 1] += ty * we;
}

}  // namespace

extern "C" void ipfem_gmsh_free(ipfem_gmsh *g)
{
    if (!g) return;
    std::free(g->xy);
    std::free(g->quads);
    std::free(g->quad_phys);
    std::free(g->lines);
    std::free(g->line_phys);
    std::free(g->points);
    std::free(g->point_phys);
    std::free(g->phys_dim);
    std::free(g->phys_tag);
    std::free(g->tris);
    std::free(g->tri_phys);
    if (g->phys_name)
        for (int32_t i = 0; i < g->n_phys; i++) std::free(g->phys_name[i]);
    std::free(g->phys_name);
    delete g;
}

extern "C" ipfem_status ipfem_gmsh_read(const char *path, ipfem_gmsh **out)
{
    if (!path || !out) return gmsh_fail("null argument");
    *out = nullptr;
    Tokens t;
    {
        FILE *f = std::fopen(path, "rb");
        if (!f) return gmsh_fail(std::string("cannot open ") + path);
        char chunk[1 << 16];
        size_t n;
        while ((n = std::fread(chunk, 1, sizeof chunk, f)) > 0) t.buf.append(chunk, n);
        std::fclose(f);
    }
    bool have_format = false, have_nodes = false, have_elements = false;
    // (dim, entity tag) -> first physical tag
    std::unordered_map<uint64_t, int32_t> ent_phys;
    auto ent_key = [](long long dim, long long tag) { return ((uint64_t)dim << 40) ^ (uint64_t)tag; };
    std::unordered_map<long long, int32_t> node_index;
    std::vector<double> xy;
    std::vector<int32_t> quads, quad_phys, lines, line_phys, points, point_phys, tris, tri_phys, pdim, ptag;
    std::vector<std::string> pname;
    while (true) {
        t.skip_ws();
        if (t.pos >= t.buf.size()) break;
        const std::string sec = t.word();
        if (sec.empty() || sec[0] != '$') return gmsh_fail("expected a section, found '" + sec + "'");
        const std::string name = sec.substr(1);
        if (name == "MeshFormat") {
            const std::string ver = t.word();
            const long long ftype = t.integer();
            t.integer();   // data size
            if (ver.compare(0, 3, "4.1") != 0) return gmsh_fail("format " + ver + " (4.1 is supported)");
            if (ftype != 0) return gmsh_fail("binary files are not supported");
            have_format = true;
        } else if (name == "PhysicalNames") {
            const long long n = t.integer();
            t.rest_of_line();
            for (long long i = 0; i < n && !t.bad; i++) {
                pdim.push_back((int32_t)t.integer());
                ptag.push_back((int32_t)t.integer());
                std::string s = t.rest_of_line();
                const size_t a = s.find('"'), b = s.rfind('"');
                pname.push_back(a != std::string::npos && b > a ? s.substr(a + 1, b - a - 1) : s);
            }
        } else if (name == "Entities") {
            long long cnt[4];
            for (int d = 0; d < 4; d++) cnt[d] = t.integer();
            for (int d = 0; d < 4 && !t.bad; d++)
                for (long long i = 0; i < cnt[d] && !t.bad; i++) {
                    const long long tag = t.integer();
                    for (int k = 0; k < (d == 0 ? 3 : 6); k++) t.real();
                    const long long np = t.integer();
                    int32_t phys = 0;
                    for (long long k = 0; k < np; k++) {
                        const long long ph = t.integer();
                        if (k == 0) phys = (int32_t)ph;
                    }
                    if (d > 0) {
                        const long long nb = t.integer();
                        for (long long k = 0; k < nb; k++) t.integer();
                    }
                    ent_phys[ent_key(d, tag)] = phys;
                }
        } else if (name == "Nodes") {
            const long long nblocks = t.integer(), nnodes = t.integer();
            t.integer();
            t.integer();
            if (t.bad || nnodes < 0 || nnodes > INT32_MAX / 2) return gmsh_fail("bad $Nodes header");
            xy.reserve((size_t)nnodes * 2);
            for (long long b = 0; b < nblocks && !t.bad; b++) {
                const long long edim = t.integer();
                t.integer();
                const long long parametric = t.integer(), n = t.integer();
                if (t.bad || n < 0 || edim < 0 || edim > 3) return gmsh_fail("bad node block");
                std::vector<long long> tags((size_t)n);
                for (long long i = 0; i < n; i++) tags[(size_t)i] = t.integer();
                for (long long i = 0; i < n && !t.bad; i++) {
                    const double x = t.real(), y = t.real(), z = t.real();
                    if (parametric) for (long long k = 0; k < edim; k++) t.real();
                    if (z != 0.0) return gmsh_fail("node outside the z = 0 plane");
                    if (!node_index.emplace(tags[(size_t)i], (int32_t)(xy.size() / 2)).second)
                        return gmsh_fail("duplicate node tag " + std::to_string(tags[(size_t)i]));
                    xy.push_back(x);
                    xy.push_back(y);
                }
            }
            have_nodes = true;
        } else if (name == "Elements") {
            if (!have_nodes) return gmsh_fail("$Elements before $Nodes");
            const long long nblocks = t.integer();
            t.integer();
            t.integer();
            t.integer();
            for (long long b = 0; b < nblocks && !t.bad; b++) {
                const long long edim = t.integer(), etag = t.integer(), type = t.integer(), n = t.integer();
                if (t.bad || n < 0) return gmsh_fail("bad element block");
                int nn;
                std::vector<int32_t> *conn, *phys;
                if (type == 15) { nn = 1; conn = &points; phys = &point_phys; }
                else if (type == 1) { nn = 2; conn = &lines; phys = &line_phys; }
                else if (type == 3) { nn = 4; conn = &quads; phys = &quad_phys; }
                else if (type == 2) { nn = 3; conn = &tris; phys = &tri_phys; }
                else
                    return gmsh_fail("element type " + std::to_string(type) +
                                     " is not supported (4-node quadrilaterals, 3-node triangles, 2-node lines "
                                     "and points)");
                auto it = ent_phys.find(ent_key(edim, etag));
                const int32_t ph = it == ent_phys.end() ? 0 : it->second;
                for (long long i = 0; i < n && !t.bad; i++) {
                    t.integer();   // element tag
                    for (int k = 0; k < nn; k++) {
                        const long long nt = t.integer();
                        auto f = node_index.find(nt);
                        if (f == node_index.end()) return gmsh_fail("unknown node tag " + std::to_string(nt));
                        conn->push_back(f->second);
                    }
                    phys->push_back(ph);
                }
            }
            have_elements = true;
        } else {
            // sections without a bearing on the problem ($Periodic, $NodeData, ...)
            const std::string end = "$End" + name;
            const size_t e = t.buf.find(end, t.pos);
            if (e == std::string::npos) return gmsh_fail("unterminated section " + sec);
            t.pos = e;
        }
        if (t.bad) return gmsh_fail("malformed section " + sec);
        const std::string end = t.word();
        if (end != "$End" + name) return gmsh_fail("expected $End" + name + ", found '" + end + "'");
    }
    if (!have_format || !have_nodes || !have_elements) return gmsh_fail("missing $MeshFormat, $Nodes or $Elements");
    ipfem_gmsh *g = new (std::nothrow) ipfem_gmsh();
    if (!g) return IPFEM_OOM;
    std::memset(g, 0, sizeof *g);
    g->n_nodes = (int32_t)(xy.size() / 2);
    g->xy = (double *)std::malloc((xy.size() ? xy.size() : 1) * sizeof(double));
    if (g->xy && !xy.empty()) std::memcpy(g->xy, xy.data(), xy.size() * sizeof(double));
    g->n_quads = (int32_t)quad_phys.size();
    g->quads = dup_i32(quads);
    g->quad_phys = dup_i32(quad_phys);
    g->n_lines = (int32_t)line_phys.size();
    g->lines = dup_i32(lines);
    g->line_phys = dup_i32(line_phys);
    g->n_points = (int32_t)point_phys.size();
    g->points = dup_i32(points);
    g->point_phys = dup_i32(point_phys);
    g->n_tris = (int32_t)tri_phys.size();
    g->tris = dup_i32(tris);
    g->tri_phys = dup_i32(tri_phys);
    g->n_phys = (int32_t)pname.size();
    g->phys_dim = dup_i32(pdim);
    g->phys_tag = dup_i32(ptag);
    g->phys_name = (char **)std::calloc(pname.size() ? pname.size() : 1, sizeof(char *));
    bool ok = g->xy && g->quads && g->quad_phys && g->lines && g->line_phys && g->points && g->point_phys &&
              g->phys_dim && g->phys_tag && g->phys_name && g->tris && g->tri_phys;
    for (size_t i = 0; ok && i < pname.size(); i++) {
        g->phys_name[i] = (char *)std::malloc(pname[i].size() + 1);
        if (!g->phys_name[i]) ok = false;
        else std::memcpy(g->phys_name[i], pname[i].c_str(), pname[i].size() + 1);
    }
    if (!ok) {
        ipfem_gmsh_free(g);
        return IPFEM_OOM;
    }
    *out = g;
    return IPFEM_OK;
}

extern "C" ipfem_status ipfem_gmsh_problem(const ipfem_gmsh *g, int32_t order, int32_t domain_phys,
                                           const ipfem_bc *bcs, int32_t n_bc, const ipfem_material *mat,
                                           ipfem_wellbore **out)
{
    if (!g || !mat || !out || (n_bc > 0 && !bcs) || n_bc < 0) return gmsh_fail("null argument");
    *out = nullptr;
    const int p = order == 0 ? 2 : order;
    if (p < 1 || p > IPFEM_MAX_ORDER) return gmsh_fail("element order must be 1, 2 or 3");
    const int nn = (p + 1) * (p + 1), ne1 = p - 1;      // connects per element, per edge interior
    if (mat->el_cohesion || mat->el_phi) return gmsh_fail("per-element material arrays are not supported here");
    for (int32_t b = 0; b < n_bc; b++) {
        const int ty = bcs[b].type;
        if (ty != 0 && ty != 1 && ty != 3 && ty != 6)
            return gmsh_fail("boundary condition type " + std::to_string(ty) + " (0, 1, 3 and 6 are supported)");
        if (ty == 0 && (bcs[b].val[0] != 0.0 || bcs[b].val[1] != 0.0))
            return gmsh_fail("non-zero Dirichlet values are not supported");
    }
    // the domain's quadrilaterals, then its triangles, in file order
    struct El {
        const int32_t *v;
        int nv;
    };
    std::vector<El> els;
    for (int32_t q = 0; q < g->n_quads; q++)
        if (domain_phys < 0 || g->quad_phys[q] == domain_phys) els.push_back({&g->quads[4 * (size_t)q], 4});
    for (int32_t q = 0; q < g->n_tris; q++)
        if (domain_phys < 0 || g->tri_phys[q] == domain_phys) els.push_back({&g->tris[3 * (size_t)q], 3});
    if (els.empty()) return gmsh_fail("no element carries physical tag " + std::to_string(domain_phys));
    const int64_t n_el = (int64_t)els.size();
    const int nt = (p + 1) * (p + 2) / 2;                // connects of a triangle
    // edges: key -> edge index; first element and number of elements per edge
    std::unordered_map<uint64_t, int32_t> edge_of;
    edge_of.reserve((size_t)n_el * 2);
    std::vector<int32_t> edge_el, edge_uses;
    std::vector<int32_t> el_edge((size_t)n_el * 4, -1);
    for (int64_t e = 0; e < n_el; e++) {
        const El &E = els[(size_t)e];
        for (int k = 0; k < E.nv; k++) {
            const int32_t a = E.v[k], b = E.v[(k + 1) % E.nv];
            if (a == b) return gmsh_fail("degenerate element");
            auto ins = edge_of.emplace(edge_key(a, b), (int32_t)edge_el.size());
            if (ins.second) {
                edge_el.push_back((int32_t)e);
                edge_uses.push_back(0);
            }
            if (++edge_uses[(size_t)ins.first->second] > 2)
                return gmsh_fail("an edge is shared by more than two elements");
            el_edge[4 * (size_t)e + k] = ins.first->second;
        }
    }
    const int64_t n_edges = (int64_t)edge_el.size();
    const int64_t n_nodes_max = (int64_t)g->n_nodes + n_edges * ne1 + n_el * nn;
    if (2 * n_nodes_max > INT32_MAX || n_el * nn * nn > INT32_MAX) return gmsh_fail("mesh too large");
    // connects numbered in order of first use by the elements; the interior
    // connects of a shared edge are numbered from its lower-numbered vertex
    std::vector<int32_t> vnew((size_t)g->n_nodes, -1), enew((size_t)(n_edges * ne1), -1);
    std::vector<int32_t> conn((size_t)n_el * nn);
    std::vector<uint8_t> ghost;                          // per connect: 1 = ghost of a triangle
    int32_t next = 0;
    auto fresh = [&](uint8_t is_ghost) {
        ghost.push_back(is_ghost);
        return next++;
    };
    for (int64_t e = 0; e < n_el; e++) {
        const El &E = els[(size_t)e];
        int32_t *c = &conn[(size_t)nn * e];
        for (int k = 0; k < E.nv; k++) {
            if (vnew[(size_t)E.v[k]] < 0) vnew[(size_t)E.v[k]] = fresh(0);
            c[k] = vnew[(size_t)E.v[k]];
        }
        for (int k = 0; k < E.nv; k++) {
            const int32_t ed = el_edge[4 * (size_t)e + k];
            const bool fwd = E.v[k] < E.v[(k + 1) % E.nv];
            for (int i = 1; i <= ne1; i++) {
                const int j = fwd ? i : p - i;          // position from the lower vertex
                int32_t &en = enew[(size_t)ed * ne1 + (j - 1)];
                if (en < 0) en = fresh(0);
                c[E.nv + k * ne1 + (i - 1)] = en;
            }
        }
        const int first_inner = E.nv + E.nv * ne1, n_real = E.nv == 4 ? nn : nt;
        for (int k = first_inner; k < n_real; k++) c[k] = fresh(0);
        for (int k = n_real; k < nn; k++) c[k] = fresh(1);
    }
    const int64_t n_nodes = next, neq = 2 * n_nodes;
    ipfem_wellbore *w = new (std::nothrow) ipfem_wellbore();
    if (!w) return IPFEM_OOM;
    std::memset(w, 0, sizeof *w);
    w->node_xy = (double *)std::calloc((size_t)n_nodes * 2, sizeof(double));
    w->connects = (int32_t *)std::calloc((size_t)n_el * nn, sizeof(int32_t));
    w->dphi = (double *)std::calloc((size_t)n_el * nn * 2 * nn, sizeof(double));
    w->weight = (double *)std::calloc((size_t)n_el * nn, sizeof(double));
    w->f0 = (double *)std::calloc((size_t)neq, sizeof(double));
    w->df = (double *)std::calloc((size_t)neq, sizeof(double));
    w->fixed = (uint8_t *)std::calloc((size_t)neq, 1);
    w->el_shape = (uint8_t *)std::calloc((size_t)n_el, 1);
    if (!w->node_xy || !w->connects || !w->dphi || !w->weight || !w->f0 || !w->df || !w->fixed || !w->el_shape) {
        ipfem_wellbore_free(w);
        return IPFEM_OOM;
    }
    std::memcpy(w->connects, conn.data(), conn.size() * sizeof(int32_t));
    for (int64_t e = 0; e < n_el; e++) w->el_shape[e] = els[(size_t)e].nv == 3;
    // coordinates: vertices, equally spaced edge connects, interior connects on
    // the bilinear (quadrilateral) or affine (triangle) map; ghosts at the
    // triangle's centre (order 2 quadrilaterals: the straight-edge midpoints
    // and the centre)
    for (int64_t e = 0; e < n_el; e++) {
        const El &E = els[(size_t)e];
        const int32_t *c = &conn[(size_t)nn * e];
        const double *pv[4];
        for (int k = 0; k < E.nv; k++) {
            pv[k] = &g->xy[2 * (size_t)E.v[k]];
            w->node_xy[2 * (size_t)c[k]] = pv[k][0];
            w->node_xy[2 * (size_t)c[k] + 1] = pv[k][1];
        }
        for (int k = 0; k < E.nv; k++) {
            const int32_t va = E.v[k], vb = E.v[(k + 1) % E.nv];
            const double *lo = &g->xy[2 * (size_t)std::min(va, vb)], *hi = &g->xy[2 * (size_t)std::max(va, vb)];
            const int32_t ed = el_edge[4 * (size_t)e + k];
            for (int j = 1; j <= ne1; j++) {
                const int32_t node = enew[(size_t)ed * ne1 + (j - 1)];
                for (int d = 0; d < 2; d++)
                    w->node_xy[2 * (size_t)node + d] = p == 2 ? 0.5 * (lo[d] + hi[d])
                                                              : (lo[d] * (p - j) + hi[d] * j) / p;
            }
        }
        const int first_inner = E.nv + E.nv * ne1;
        for (int k = first_inner; k < nn; k++) {
            for (int d = 0; d < 2; d++) {
                double x;
                if (E.nv == 3) {
                    x = (pv[0][d] + pv[1][d] + pv[2][d]) / 3.0;     // interior node (order 3) and ghosts
                } else if (p == 2) {
                    x = 0.25 * (((pv[0][d] + pv[1][d]) + pv[2][d]) + pv[3][d]);
                } else {
                    const int m = k - first_inner, ia = m % ne1 + 1, ib = m / ne1 + 1;
                    const double u = (double)ia / p, t = (double)ib / p;
                    x = (1.0 - u) * (1.0 - t) * pv[0][d] + u * (1.0 - t) * pv[1][d] + u * t * pv[2][d] +
                        (1.0 - u) * t * pv[3][d];
                }
                w->node_xy[2 * (size_t)c[k] + d] = x;
            }
        }
    }
    element_blocks_dphi(p, n_el, w->connects, w->node_xy, w->dphi, w->weight, w->el_shape);
    for (int64_t i = 0; i < n_nodes; i++)
        if (ghost[(size_t)i]) {
            w->fixed[2 * (size_t)i] = w->fixed[2 * (size_t)i + 1] = 1;
            w->n_ghost++;
        }
    // boundary conditions
    for (int32_t b = 0; b < n_bc; b++) {
        const ipfem_bc &bc = bcs[b];
        int64_t hits = 0;
        auto fix_node = [&](int32_t node) {
            for (int k = 0; k < 2; k++)
                if (bc.type == 0 || bc.val[k] != 0.0) w->fixed[2 * (size_t)node + k] = 1;
        };
        for (int32_t l = 0; l < g->n_lines; l++) {
            if (g->line_phys[l] != bc.phys) continue;
            hits++;
            const int32_t a = g->lines[2 * (size_t)l], bb = g->lines[2 * (size_t)l + 1];
            auto f = edge_of.find(edge_key(a, bb));
            if (f == edge_of.end()) {
                ipfem_wellbore_free(w);
                return gmsh_fail("a line of physical tag " + std::to_string(bc.phys) + " is not an element edge");
            }
            const int32_t ed = f->second;
            const int32_t A = vnew[(size_t)std::min(a, bb)], B = vnew[(size_t)std::max(a, bb)];
            // connects of the line from its lower vertex: A, edge connects, B
            std::vector<int32_t> line_nodes;
            line_nodes.push_back(A);
            for (int j = 1; j <= ne1; j++) line_nodes.push_back(enew[(size_t)ed * ne1 + (j - 1)]);
            line_nodes.push_back(B);
            if (bc.type == 0 || bc.type == 3) {
                for (int32_t node : line_nodes) fix_node(node);
                continue;
            }
            double tx = bc.val[0], ty = bc.val[1];
            if (bc.type == 6) {
                if (edge_uses[(size_t)ed] != 1) {
                    ipfem_wellbore_free(w);
                    return gmsh_fail("a normal-stress line of physical tag " + std::to_string(bc.phys) +
                                     " is not on the boundary");
                }
                // outward normal: away from the adjacent element's vertex centre
                const double *pa = &w->node_xy[2 * (size_t)A], *pb = &w->node_xy[2 * (size_t)B];
                const double dx = pb[0] - pa[0], dy = pb[1] - pa[1];
                const double L = std::sqrt(dx * dx + dy * dy);
                double nx = dy / L, ny = -dx / L;
                const El &Ea = els[(size_t)edge_el[(size_t)ed]];
                double cx = 0.0, cy = 0.0;
                for (int k = 0; k < Ea.nv; k++) {
                    cx += g->xy[2 * (size_t)Ea.v[k]] / Ea.nv;
                    cy += g->xy[2 * (size_t)Ea.v[k] + 1] / Ea.nv;
                }
                if ((cx - 0.5 * (pa[0] + pb[0])) * nx + (cy - 0.5 * (pa[1] + pb[1])) * ny > 0.0) {
                    nx = -nx;
                    ny = -ny;
                }
                tx = bc.val[0] * nx;
                ty = bc.val[0] * ny;
            }
            if (p == 2) {
                edge_load(w->node_xy, A, line_nodes[1], B, tx, ty, w->df);
            } else {
                // consistent load of a constant traction: the order-p Lagrange trace
                // functions on equispaced nodes integrate to L/2 (p = 1) and
                // L/8, 3L/8, 3L/8, L/8 (p = 3)
                const double *pa = &w->node_xy[2 * (size_t)A], *pb = &w->node_xy[2 * (size_t)B];
                const double dx = pb[0] - pa[0], dy = pb[1] - pa[1];
                const double L = std::sqrt(dx * dx + dy * dy);
                const double w1[2] = {0.5, 0.5}, w3[4] = {0.125, 0.375, 0.375, 0.125};
                for (int k = 0; k <= p; k++) {
                    const double wk = (p == 1 ? w1[k] : w3[k]) * L;
                    w->df[2 * (size_t)line_nodes[(size_t)k]] += tx * wk;
                    w->df[2 * (size_t)line_nodes[(size_t)k] + 1] += ty * wk;
                }
            }
        }
        for (int32_t q = 0; q < g->n_points; q++) {
            if (g->point_phys[q] != bc.phys) continue;
            hits++;
            const int32_t node = vnew[(size_t)g->points[q]];
            if (node < 0) {
                ipfem_wellbore_free(w);
                return gmsh_fail("a point of physical tag " + std::to_string(bc.phys) + " is not an element vertex");
            }
            if (bc.type == 1 || bc.type == 6) {
                ipfem_wellbore_free(w);
                return gmsh_fail("traction boundary conditions need lines (physical tag " + std::to_string(bc.phys) +
                                 " has points)");
            }
            fix_node(node);
        }
        if (hits == 0) {
            ipfem_wellbore_free(w);
            return gmsh_fail("no line or point carries physical tag " + std::to_string(bc.phys));
        }
    }
    w->material = *mat;
    w->material.el_cohesion = nullptr;
    w->material.el_phi = nullptr;
    w->mesh.n_elements = (int32_t)n_el;
    w->mesh.n_nodes = (int32_t)n_nodes;
    w->mesh.connects = w->connects;
    w->mesh.dphi = w->dphi;
    w->mesh.block_storage = nullptr;
    w->mesh.weight = w->weight;
    w->mesh.fixed = w->fixed;
    w->mesh.f0 = w->f0;
    w->mesh.df = w->df;
    w->mesh.order = p;
    *out = w;
    return IPFEM_OK;
}
