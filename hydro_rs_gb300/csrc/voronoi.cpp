// Host Voronoi mesh builder: generators -> face list + cell->face CSR.
//
// The reference builds its mesh with the meshless_voronoi crate (0.6.1, called
// from src/space.rs:571-594 and :236-263); that crate is not part of the hot
// path and is not vendored, so this file is this library's own builder.  It
// produces the same quantities the reference's flux/gradient code consumes:
//   face: left, right (or -1 for a wall), area, unit normal (left -> right /
//         outward), centroid, periodic shift of the right cell's image;
//   cell: volume, centroid, and the CSR list of face indices.
// Conventions (matching the reference's consumers, src/flux.rs:34-38,
// src/runner/hydrodynamics.rs:84-85): a face is owned by the lower cell index
// (left = i < right = j); a periodic face stores right = the real index j and
// shift = offset of the image of j adjacent to i.  Lower-dimensional runs use
// unit extent along unused axes, so 1D faces have area 1 and 2D face "area" is
// the edge length.
//
// Algorithm: each cell is the box (or a large square/cube for periodic runs)
// clipped by the bisector half-spaces of nearby generators, found ring by ring
// in a uniform bin grid, until the security radius criterion (next ring at
// distance >= 2 * max vertex distance) holds.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct P3 {
    double x, y, z;
};
inline P3 operator+(P3 a, P3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline P3 operator-(P3 a, P3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline P3 operator*(double s, P3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline P3 cross(P3 a, P3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double norm(P3 a) { return std::sqrt(dot(a, a)); }

// Edge / face labels: >= 0 neighbour generator (with shift index), walls
// encoded negative: -1 x-, -2 x+, -3 y-, -4 y+, -5 z-, -6 z+; -100 invalid.
constexpr int64_t kInvalid = -100;

struct FaceOut {
    int64_t nb;  // neighbour index or wall code
    int sx, sy, sz;
    double area;
    P3 centroid;
};

struct CellOut {
    double volume = 0;
    P3 centroid{0, 0, 0};
    std::vector<FaceOut> faces;
    int error = 0;
};

struct Grid {
    int dim;
    int nb[3];
    double bw[3];
    double box[3];
    bool periodic;
    std::vector<int32_t> start;  // bin -> first index into order
    std::vector<int32_t> order;
    double minbw;
};

Grid make_grid(int dim, int64_t n, const double* g, const double* box, bool periodic) {
    Grid gr;
    gr.dim = dim;
    gr.periodic = periodic;
    double vol = 1;
    for (int k = 0; k < dim; k++) vol *= box[k];
    double h = std::pow(vol / double(n), 1.0 / dim);  // mean spacing
    for (int k = 0; k < 3; k++) {
        gr.box[k] = box[k];
        if (k < dim) {
            gr.nb[k] = std::max(1, int(std::floor(box[k] / h)));
            gr.bw[k] = box[k] / gr.nb[k];
        } else {
            gr.nb[k] = 1;
            gr.bw[k] = box[k];
        }
    }
    gr.minbw = gr.bw[0];
    for (int k = 1; k < dim; k++) gr.minbw = std::min(gr.minbw, gr.bw[k]);
    int64_t nbins = int64_t(gr.nb[0]) * gr.nb[1] * gr.nb[2];
    std::vector<int64_t> bin(n);
    std::vector<int32_t> cnt(nbins + 1, 0);
    for (int64_t i = 0; i < n; i++) {
        int b[3] = {0, 0, 0};
        for (int k = 0; k < dim; k++) {
            int v = int(std::floor(g[k * n + i] / gr.bw[k]));
            b[k] = std::min(std::max(v, 0), gr.nb[k] - 1);
        }
        bin[i] = (int64_t(b[0]) * gr.nb[1] + b[1]) * gr.nb[2] + b[2];
        cnt[bin[i] + 1]++;
    }
    for (int64_t b = 0; b < nbins; b++) cnt[b + 1] += cnt[b];
    gr.start.assign(cnt.begin(), cnt.end());
    gr.order.resize(n);
    std::vector<int32_t> fill(cnt.begin(), cnt.end() - 1);
    for (int64_t i = 0; i < n; i++) gr.order[fill[bin[i]]++] = int32_t(i);
    return gr;
}

// Iterate the bins at Chebyshev ring r around bin (b0,b1,b2); calls
// fn(j, shift) for every generator j in those bins (with periodic image shift
// counts in units of the box).
template <typename Fn>
void for_ring(const Grid& gr, const int b[3], int r, Fn&& fn) {
    int lo[3], hi[3];
    for (int k = 0; k < 3; k++) {
        if (k < gr.dim) { lo[k] = -r; hi[k] = r; } else { lo[k] = 0; hi[k] = 0; }
    }
    for (int dx = lo[0]; dx <= hi[0]; dx++)
        for (int dy = lo[1]; dy <= hi[1]; dy++)
            for (int dz = lo[2]; dz <= hi[2]; dz++) {
                int m = std::max(std::abs(dx), std::max(std::abs(dy), std::abs(dz)));
                if (m != r) continue;
                int c[3] = {b[0] + dx, b[1] + dy, b[2] + dz};
                int s[3] = {0, 0, 0};
                bool skip = false;
                for (int k = 0; k < gr.dim; k++) {
                    if (c[k] < 0 || c[k] >= gr.nb[k]) {
                        if (!gr.periodic) { skip = true; break; }
                        int w = ((c[k] % gr.nb[k]) + gr.nb[k]) % gr.nb[k];
                        s[k] = (c[k] - w) / gr.nb[k];
                        c[k] = w;
                    }
                }
                if (skip) continue;
                int64_t bb = (int64_t(c[0]) * gr.nb[1] + c[1]) * gr.nb[2] + c[2];
                for (int32_t q = gr.start[bb]; q < gr.start[bb + 1]; q++) fn(gr.order[q], s);
            }
}

// ----------------------------------------------------------------- 2D ----
// A convex polygon in fixed storage: a 2D Voronoi cell has a few dozen
// vertices at most, and the clipping below then allocates nothing.
constexpr int kMaxPoly2 = 128;
struct Poly2 {
    int n = 0;
    P3 v[kMaxPoly2];        // vertices (z unused)
    int64_t lab[kMaxPoly2]; // label of edge v[k] -> v[k+1]
    int sh[kMaxPoly2];      // packed shift of that edge's neighbour
    void push(P3 p, int64_t l, int s) {
        v[n] = p;
        lab[n] = l;
        sh[n] = s;
        n++;
    }
};

inline int pack_shift(const int s[3]) { return (s[0] + 8) | ((s[1] + 8) << 4) | ((s[2] + 8) << 8); }
inline void unpack_shift(int p, int s[3]) {
    s[0] = (p & 15) - 8;
    s[1] = ((p >> 4) & 15) - 8;
    s[2] = ((p >> 8) & 15) - 8;
}

// Clips P by the half-space dot(x - m, d) <= eps into Q (Q = P if nothing is
// cut); false when Q would exceed its storage.  Returns with *changed set
// when the polygon changed.
bool clip2(const Poly2& P, Poly2& Q, P3 m, P3 d, int64_t lab, int sh, double eps, bool* changed) {
    const int nv = P.n;
    double h[kMaxPoly2];
    bool any_out = false;
    for (int k = 0; k < nv; k++) {
        h[k] = dot(P.v[k] - m, d);
        if (h[k] > eps) any_out = true;
    }
    *changed = any_out;
    if (!any_out) return true;
    Q.n = 0;
    for (int k = 0; k < nv; k++) {
        if (Q.n + 2 > kMaxPoly2) return false;
        const int k1 = k + 1 == nv ? 0 : k + 1;
        const P3 a = P.v[k], b = P.v[k1];
        const bool ain = h[k] <= eps, bin = h[k1] <= eps;
        if (ain) {
            if (bin) {
                Q.push(a, P.lab[k], P.sh[k]);
            } else if (h[k] >= -eps) {
                // leaving with a on the plane: the new edge starts at a itself
                Q.push(a, lab, sh);
            } else {
                // leaving: a -> cut point keeps the old label, cut -> next entry is new
                const double t = h[k] / (h[k] - h[k1]);
                Q.push(a, P.lab[k], P.sh[k]);
                Q.push(a + t * (b - a), lab, sh);
            }
        } else if (bin) {
            // entering: cut point -> b keeps the old label
            if (h[k1] >= -eps) continue;  // b on the plane: b itself is the entry point
            const double t = h[k] / (h[k] - h[k1]);
            Q.push(a + t * (b - a), P.lab[k], P.sh[k]);
        }
    }
    return true;
}

CellOut build_cell2(int64_t i, int64_t n, const double* g, const Grid& gr) {
    CellOut out;
    P3 gi{g[i], g[n + i], 0.0};
    Poly2 buf[2];
    Poly2* P = &buf[0];
    Poly2* Q = &buf[1];
    double L0 = gr.box[0], L1 = gr.box[1];
    int zero3[3] = {0, 0, 0};
    const int sh0 = pack_shift(zero3);
    if (!gr.periodic) {
        P->push({0, 0, 0}, -3, sh0);
        P->push({L0, 0, 0}, -2, sh0);
        P->push({L0, L1, 0}, -4, sh0);
        P->push({0, L1, 0}, -1, sh0);
    } else {
        double hx = 0.5 * L0, hy = 0.5 * L1;
        P->push({gi.x - hx, gi.y - hy, 0}, kInvalid, sh0);
        P->push({gi.x + hx, gi.y - hy, 0}, kInvalid, sh0);
        P->push({gi.x + hx, gi.y + hy, 0}, kInvalid, sh0);
        P->push({gi.x - hx, gi.y + hy, 0}, kInvalid, sh0);
    }
    // the largest squared vertex distance from the generator, kept current
    auto reach2 = [&]() {
        double r2 = 0;
        for (int k = 0; k < P->n; k++) r2 = std::max(r2, dot(P->v[k] - gi, P->v[k] - gi));
        return r2;
    };
    double r2 = reach2();
    int b[3] = {std::min(std::max(int(std::floor(gi.x / gr.bw[0])), 0), gr.nb[0] - 1),
                std::min(std::max(int(std::floor(gi.y / gr.bw[1])), 0), gr.nb[1] - 1), 0};
    double eps = 1e-13 * gr.minbw * gr.minbw;
    int rmax = std::max(gr.nb[0], gr.nb[1]) + 1;
    for (int r = 0; r <= rmax; r++) {
        double reach = (r - 1) * gr.minbw;
        if (r >= 1 && reach > 0 && reach * reach >= 4.0 * r2) break;
        for_ring(gr, b, r, [&](int32_t j, const int s[3]) {
            if (j == i && s[0] == 0 && s[1] == 0) return;
            P3 gj{g[j] + s[0] * L0, g[n + j] + s[1] * L1, 0.0};
            P3 d = gj - gi;
            double dd = dot(d, d);
            if (dd >= 4.0 * r2) return;
            if (j == i) { out.error = 2; return; }
            P3 m = 0.5 * (gi + gj);
            bool changed = false;
            if (!clip2(*P, *Q, m, d, j, pack_shift(s), eps * std::sqrt(dd), &changed)) {
                out.error = 3;
                return;
            }
            if (changed) {
                std::swap(P, Q);
                r2 = reach2();
            }
        });
        if (out.error) return out;
    }
    const int nv = P->n;
    // polygon area / centroid relative to the generator
    double A = 0, cx = 0, cy = 0;
    double per = 0;
    for (int k = 0; k < nv; k++) {
        P3 a = P->v[k] - gi, c = P->v[(k + 1) % nv] - gi;
        double cr = a.x * c.y - c.x * a.y;
        A += cr;
        cx += (a.x + c.x) * cr;
        cy += (a.y + c.y) * cr;
        per += norm(c - a);
    }
    A *= 0.5;
    double Lz = gr.box[2];
    out.volume = A * Lz;
    out.centroid = {gi.x + cx / (6 * A), gi.y + cy / (6 * A), 0.5 * Lz};
    out.faces.reserve(nv);
    for (int k = 0; k < nv; k++) {
        if (P->lab[k] == kInvalid) { out.error = 1; continue; }
        P3 a = P->v[k], c = P->v[(k + 1) % nv];
        double len = norm(c - a);
        if (len <= 1e-12 * per) continue;
        FaceOut f;
        f.nb = P->lab[k];
        int s[3];
        unpack_shift(P->sh[k], s);
        f.sx = s[0]; f.sy = s[1]; f.sz = s[2];
        f.area = len * Lz;
        f.centroid = {0.5 * (a.x + c.x), 0.5 * (a.y + c.y), 0.5 * Lz};
        out.faces.push_back(f);
    }
    return out;
}

// ----------------------------------------------------------------- 3D ----
// A convex polyhedron in fixed storage: vertices, and each face a loop of
// vertex indices (counter-clockwise seen from outside) in one index array.
constexpr int kMaxV3 = 512, kMaxF3 = 160, kMaxI3 = 2048;
struct Poly3 {
    int nv = 0, nf = 0;
    P3 v[kMaxV3];
    int fo[kMaxF3 + 1];  // face k's loop is idx[fo[k] .. fo[k + 1])
    int idx[kMaxI3];
    int64_t lab[kMaxF3];
    int sh[kMaxF3];
};

void box3(Poly3& P, P3 lo, P3 hi, bool invalid) {
    const P3 v[8] = {{lo.x, lo.y, lo.z}, {hi.x, lo.y, lo.z}, {hi.x, hi.y, lo.z}, {lo.x, hi.y, lo.z},
                     {lo.x, lo.y, hi.z}, {hi.x, lo.y, hi.z}, {hi.x, hi.y, hi.z}, {lo.x, hi.y, hi.z}};
    const int f[6][4] = {{0, 3, 2, 1}, {4, 5, 6, 7}, {0, 1, 5, 4}, {2, 3, 7, 6}, {0, 4, 7, 3}, {1, 2, 6, 5}};
    const int64_t walls[6] = {-5, -6, -3, -4, -1, -2};
    int z[3] = {0, 0, 0};
    P.nv = 8;
    for (int k = 0; k < 8; k++) P.v[k] = v[k];
    P.nf = 6;
    for (int k = 0; k < 6; k++) {
        P.fo[k] = 4 * k;
        for (int j = 0; j < 4; j++) P.idx[4 * k + j] = f[k][j];
        P.lab[k] = invalid ? kInvalid : walls[k];
        P.sh[k] = pack_shift(z);
    }
    P.fo[6] = 24;
}

// Clips P by the half-space dot(x - m, d) <= eps into Q.  Returns 0 when
// nothing is cut (Q untouched), 1 when Q holds the clipped polyhedron, -1 when
// it would not fit.  Each face keeps its inside part; the cut points on the
// plane, one per crossing edge, are chained into the new face.
int clip3(const Poly3& P, Poly3& Q, P3 m, P3 d, int64_t lab, int sh, double eps) {
    const int nv = P.nv;
    double h[kMaxV3];
    bool any_out = false;
    for (int k = 0; k < nv; k++) {
        h[k] = dot(P.v[k] - m, d);
        if (h[k] > eps) any_out = true;
    }
    if (!any_out) return 0;
    int newid[kMaxV3];
    for (int k = 0; k < nv; k++) newid[k] = -1;
    Q.nv = 0;
    Q.nf = 0;
    Q.fo[0] = 0;
    bool full = false;
    auto keep = [&](int a) {  // a vertex of P that stays
        if (newid[a] < 0) {
            if (Q.nv >= kMaxV3) { full = true; return 0; }
            newid[a] = Q.nv;
            Q.v[Q.nv++] = P.v[a];
        }
        return newid[a];
    };
    // the cut point of edge (a inside, b outside), one per edge
    uint64_t cut_key[kMaxF3];
    int cut_id[kMaxF3], ncut = 0;
    auto edge_point = [&](int a, int b) -> int {
        if (h[a] >= -eps && h[a] <= eps) return keep(a);  // a lies on the plane
        const uint64_t key = (uint64_t(std::min(a, b)) << 32) | uint64_t(std::max(a, b));
        for (int k = 0; k < ncut; k++)
            if (cut_key[k] == key) return cut_id[k];
        if (ncut >= kMaxF3 || Q.nv >= kMaxV3) { full = true; return 0; }
        const double t = h[a] / (h[a] - h[b]);
        Q.v[Q.nv] = P.v[a] + t * (P.v[b] - P.v[a]);
        cut_key[ncut] = key;
        cut_id[ncut++] = Q.nv;
        return Q.nv++;
    };
    int chain_from[kMaxF3], chain_to[kMaxF3], nchain = 0;  // on the cut plane: entry -> exit
    for (int fi = 0; fi < P.nf && !full; fi++) {
        const int f0 = P.fo[fi], mlen = P.fo[fi + 1] - f0;
        const int start = Q.fo[Q.nf];
        int len = 0, exitp = -1, entryp = -1;
        auto push = [&](int x) {
            if (start + len >= kMaxI3) { full = true; return; }
            Q.idx[start + len++] = x;
        };
        for (int k = 0; k < mlen; k++) {
            const int a = P.idx[f0 + k], b = P.idx[f0 + (k + 1 == mlen ? 0 : k + 1)];
            const bool ain = h[a] <= eps, bin = h[b] <= eps;
            if (ain) {
                const int qa = keep(a);
                push(qa);
                if (!bin) {
                    const int p = edge_point(a, b);
                    if (p != qa) push(p);
                    exitp = p;
                }
            } else if (bin) {
                const int p = edge_point(b, a);
                const bool b_on_plane = h[b] >= -eps && h[b] <= eps;
                if (!b_on_plane) push(p);
                entryp = p;
            }
        }
        if (exitp >= 0 && entryp >= 0 && exitp != entryp) {
            if (nchain >= kMaxF3) { full = true; break; }
            chain_from[nchain] = entryp;
            chain_to[nchain++] = exitp;
        }
        if (len >= 3) {
            if (Q.nf >= kMaxF3) { full = true; break; }
            Q.lab[Q.nf] = P.lab[fi];
            Q.sh[Q.nf] = P.sh[fi];
            Q.fo[++Q.nf] = start + len;
        }
    }
    if (full) return -1;
    // the new face: each clipped face contributes entry -> exit along the cut
    if (nchain > 0) {
        const int start = Q.fo[Q.nf];
        int len = 0;
        const int first = chain_from[0];
        int cur = first;
        bool closed = false;
        for (int guard = 0; guard <= nchain + 1; guard++) {
            if (start + len >= kMaxI3) return -1;
            Q.idx[start + len++] = cur;
            int nx = -1;
            for (int k = 0; k < nchain; k++)
                if (chain_from[k] == cur) { nx = chain_to[k]; break; }
            if (nx < 0) break;
            cur = nx;
            if (cur == first) { closed = true; break; }
        }
        if (closed && len >= 3) {
            if (Q.nf >= kMaxF3) return -1;
            Q.lab[Q.nf] = lab;
            Q.sh[Q.nf] = sh;
            Q.fo[++Q.nf] = start + len;
        }
    }
    // drop the vertices no face uses (in order: a vertex moves to a lower slot)
    int used[kMaxV3];
    for (int k = 0; k < Q.nv; k++) used[k] = -1;
    const int nidx = Q.fo[Q.nf];
    for (int k = 0; k < nidx; k++) used[Q.idx[k]] = 0;
    int nn = 0;
    for (int k = 0; k < Q.nv; k++)
        if (used[k] == 0) {
            used[k] = nn;
            Q.v[nn++] = Q.v[k];
        }
    Q.nv = nn;
    for (int k = 0; k < nidx; k++) Q.idx[k] = used[Q.idx[k]];
    return 1;
}

CellOut build_cell3(int64_t i, int64_t n, const double* g, const Grid& gr) {
    CellOut out;
    P3 gi{g[i], g[n + i], g[2 * n + i]};
    static thread_local Poly3 buf[2];
    Poly3* P = &buf[0];
    Poly3* Q = &buf[1];
    double L[3] = {gr.box[0], gr.box[1], gr.box[2]};
    if (!gr.periodic) box3(*P, {0, 0, 0}, {L[0], L[1], L[2]}, false);
    else box3(*P, gi - P3{0.5 * L[0], 0.5 * L[1], 0.5 * L[2]}, gi + P3{0.5 * L[0], 0.5 * L[1], 0.5 * L[2]}, true);
    int b[3];
    for (int k = 0; k < 3; k++) {
        double c = k == 0 ? gi.x : (k == 1 ? gi.y : gi.z);
        b[k] = std::min(std::max(int(std::floor(c / gr.bw[k])), 0), gr.nb[k] - 1);
    }
    double eps = 1e-13 * gr.minbw * gr.minbw;
    int rmax = std::max(gr.nb[0], std::max(gr.nb[1], gr.nb[2])) + 1;
    auto reach2 = [&]() {
        double r2 = 0;
        for (int k = 0; k < P->nv; k++) r2 = std::max(r2, dot(P->v[k] - gi, P->v[k] - gi));
        return r2;
    };
    double r2max = reach2();
    static thread_local std::vector<std::pair<double, std::pair<int32_t, int>>> cand;
    for (int r = 0; r <= rmax; r++) {
        double reach = (r - 1) * gr.minbw;
        if (r >= 1 && reach > 0 && reach * reach >= 4.0 * r2max) break;
        // this ring's candidates sorted by distance: nearer planes cut more
        cand.clear();
        for_ring(gr, b, r, [&](int32_t j, const int s[3]) {
            if (j == i && s[0] == 0 && s[1] == 0 && s[2] == 0) return;
            P3 gj{g[j] + s[0] * L[0], g[n + j] + s[1] * L[1], g[2 * n + j] + s[2] * L[2]};
            P3 d = gj - gi;
            cand.push_back({dot(d, d), {j, pack_shift(s)}});
        });
        std::sort(cand.begin(), cand.end());
        for (auto& c : cand) {
            if (c.first >= 4.0 * r2max) break;
            int32_t j = c.second.first;
            int s[3];
            unpack_shift(c.second.second, s);
            if (j == i) { out.error = 2; continue; }
            P3 gj{g[j] + s[0] * L[0], g[n + j] + s[1] * L[1], g[2 * n + j] + s[2] * L[2]};
            P3 d = gj - gi;
            const int rc = clip3(*P, *Q, 0.5 * (gi + gj), d, j, c.second.second, eps * std::sqrt(c.first));
            if (rc < 0) {
                out.error = 3;
                return out;
            }
            if (rc > 0) {
                std::swap(P, Q);
                r2max = reach2();
            }
        }
    }
    // integrals: faces by fan triangulation, volume by tetrahedra from gi
    double V = 0;
    P3 C{0, 0, 0};
    double total_area = 0;
    double fa[kMaxF3];
    P3 fc[kMaxF3];
    for (int fi = 0; fi < P->nf; fi++) {
        const int* F = P->idx + P->fo[fi];
        const int len = P->fo[fi + 1] - P->fo[fi];
        P3 a0 = P->v[F[0]] - gi;
        double A = 0;
        P3 ac{0, 0, 0};
        for (int k = 1; k + 1 < len; k++) {
            P3 a1 = P->v[F[k]] - gi, a2 = P->v[F[k + 1]] - gi;
            P3 cr = cross(a1 - a0, a2 - a0);
            double ta = 0.5 * norm(cr);
            A += ta;
            ac = ac + (ta / 3.0) * (a0 + a1 + a2);
            double tv = dot(a0, cross(a1, a2)) / 6.0;
            V += tv;
            C = C + (tv / 4.0) * (a0 + a1 + a2);
        }
        fa[fi] = A;
        fc[fi] = A > 0 ? gi + (1.0 / A) * ac : gi + a0;
        total_area += A;
    }
    out.volume = V;
    out.centroid = gi + (1.0 / V) * C;
    out.faces.reserve(P->nf);
    for (int fi = 0; fi < P->nf; fi++) {
        if (P->lab[fi] == kInvalid) { out.error = 1; continue; }
        if (fa[fi] <= 1e-12 * total_area) continue;
        FaceOut f;
        f.nb = P->lab[fi];
        int s[3];
        unpack_shift(P->sh[fi], s);
        f.sx = s[0]; f.sy = s[1]; f.sz = s[2];
        f.area = fa[fi];
        f.centroid = fc[fi];
        out.faces.push_back(f);
    }
    return out;
}

struct Built {
    int64_t n = 0;
    std::vector<int32_t> left, right, csr_off, csr_face;
    std::vector<double> area, normal, centroid, shift, volume, cell_centroid;
};

}  // namespace

extern "C" {

// Builds the mesh.  gen is [3][n]; box[3]; returns 0 on success, writes the
// face count and an opaque handle.
int mvmm_voronoi_build(int dim, int64_t n, const double* gen, const double* box, int periodic, int n_threads,
                       int64_t* n_faces, void** handle) {
    if (dim != 2 && dim != 3) return -1;
    if (n <= 0) return -2;
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
    Grid gr = make_grid(dim, n, gen, box, periodic != 0);
    if (periodic)
        for (int k = 0; k < dim; k++)
            if (gr.nb[k] < 3) return -3;  // a cell could neighbour its own image
    std::vector<CellOut> cells(n);
    int err = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(| : err)
    for (int64_t i = 0; i < n; i++) {
        cells[i] = dim == 2 ? build_cell2(i, n, gen, gr) : build_cell3(i, n, gen, gr);
        err |= cells[i].error;
    }
    if (err) return -10 - err;
    // Faces are owned by the lower cell index (or are walls) and numbered in
    // owner order, then in the owner's own order; every cell lists its faces
    // in increasing index.  Each part runs over the cells in parallel.
    Built* B = new Built();
    B->n = n;
    B->volume.resize(n);
    B->cell_centroid.resize(3 * n);
    std::vector<int64_t> first(n + 1, 0);  // the first face each cell owns
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        B->volume[i] = cells[i].volume;
        B->cell_centroid[i] = cells[i].centroid.x;
        B->cell_centroid[n + i] = cells[i].centroid.y;
        B->cell_centroid[2 * n + i] = cells[i].centroid.z;
        int64_t c = 0;
        for (auto& f : cells[i].faces)
            if (f.nb < 0 || f.nb > i) c++;
        first[i + 1] = c;
    }
    for (int64_t i = 0; i < n; i++) first[i + 1] += first[i];
    const int64_t nf = first[n];
    B->left.resize(nf);
    B->right.resize(nf);
    B->area.resize(nf);
    B->normal.resize(3 * nf);
    B->centroid.resize(3 * nf);
    B->shift.resize(3 * nf);
    std::vector<int32_t> deg(n, 0);  // faces per cell
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        P3 gi{gen[i], gen[n + i], gen[2 * n + i]};
        int64_t idx = first[i];
        for (auto& f : cells[i].faces) {
            if (f.nb >= 0 && f.nb <= i) continue;
            B->left[idx] = int32_t(i);
            B->area[idx] = f.area;
            B->centroid[idx] = f.centroid.x;
            B->centroid[nf + idx] = f.centroid.y;
            B->centroid[2 * nf + idx] = f.centroid.z;
            P3 nn{0, 0, 0}, s{0, 0, 0};
            if (f.nb >= 0) {
                int64_t j = f.nb;
                s = P3{f.sx * box[0], f.sy * box[1], f.sz * box[2]};
                P3 gj{gen[j] + s.x, gen[n + j] + s.y, gen[2 * n + j] + s.z};
                P3 d = gj - gi;
                nn = (1.0 / norm(d)) * d;
                B->right[idx] = int32_t(j);
#pragma omp atomic
                deg[j]++;
            } else {
                if (f.nb == -1) nn.x = -1; else if (f.nb == -2) nn.x = 1;
                else if (f.nb == -3) nn.y = -1; else if (f.nb == -4) nn.y = 1;
                else if (f.nb == -5) nn.z = -1; else nn.z = 1;
                B->right[idx] = -1;
            }
            B->normal[idx] = nn.x;
            B->normal[nf + idx] = nn.y;
            B->normal[2 * nf + idx] = nn.z;
            B->shift[idx] = s.x;
            B->shift[nf + idx] = s.y;
            B->shift[2 * nf + idx] = s.z;
            idx++;
        }
    }
    B->csr_off.resize(n + 1);
    B->csr_off[0] = 0;
    for (int64_t i = 0; i < n; i++)
        B->csr_off[i + 1] = B->csr_off[i] + int32_t(first[i + 1] - first[i]) + deg[i];
    B->csr_face.resize(B->csr_off[n]);
    std::vector<int32_t> fill(B->csr_off.begin(), B->csr_off.end() - 1);
#pragma omp parallel for schedule(static)
    for (int64_t f = 0; f < nf; f++) {
        int32_t slot;
#pragma omp atomic capture
        slot = fill[B->left[f]]++;
        B->csr_face[slot] = int32_t(f);
        const int32_t j = B->right[f];
        if (j >= 0) {
#pragma omp atomic capture
            slot = fill[j]++;
            B->csr_face[slot] = int32_t(f);
        }
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) std::sort(B->csr_face.begin() + B->csr_off[i], B->csr_face.begin() + B->csr_off[i + 1]);
    *n_faces = nf;
    *handle = B;
    return 0;
}

int mvmm_voronoi_fetch(void* handle, int32_t* left, int32_t* right, double* area, double* normal, double* centroid,
                       double* shift, int32_t* csr_off, int32_t* csr_face, double* volume, double* cell_centroid) {
    Built* B = static_cast<Built*>(handle);
    size_t nf = B->left.size();
    std::memcpy(left, B->left.data(), nf * 4);
    std::memcpy(right, B->right.data(), nf * 4);
    std::memcpy(area, B->area.data(), nf * 8);
    std::memcpy(normal, B->normal.data(), 3 * nf * 8);
    std::memcpy(centroid, B->centroid.data(), 3 * nf * 8);
    std::memcpy(shift, B->shift.data(), 3 * nf * 8);
    std::memcpy(csr_off, B->csr_off.data(), (B->n + 1) * 4);
    std::memcpy(csr_face, B->csr_face.data(), B->csr_face.size() * 4);
    std::memcpy(volume, B->volume.data(), B->n * 8);
    std::memcpy(cell_centroid, B->cell_centroid.data(), 3 * B->n * 8);
    return 0;
}

void mvmm_voronoi_free(void* handle) { delete static_cast<Built*>(handle); }

}  // extern "C"
