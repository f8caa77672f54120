// Host-side set-up of the clustering seam (plain C++, no device code): the
// reference's edge numbering and vertex rings, the metric plugins' vertex
// weights and the default initial sampling.  These run before
// MinimizeEnergy() in the reference too (Init / BuildMetric / InitSamples,
// Common/vtkUniformClustering.h:1363,1124) and are not part of the GPU hot path.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <queue>
#include <random>
#include <unordered_map>
#include <vector>

#include "../../include/acvd_gpu.h"

namespace {

// Edge table in the reference's numbering (vtkSurfaceBase::AddEdge,
// Common/vtkSurfaceBase.cxx:1166-1221, driven by CreateFromPolyData :1407-1468):
// faces are scanned in order; the pair (v_j, v_j+1) becomes a new edge the first
// time it is seen; the first two faces using an edge are its Poly1 / Poly2.
struct EdgeTable {
    int64_t nv = 0;
    std::vector<int32_t> v1, v2, poly1, poly2;
    std::vector<std::pair<int32_t, int32_t>> extra_faces;   // (edge, face) beyond two faces
    std::vector<int64_t> ring_row;                           // ring CSR (edge ids, creation order)
    std::vector<int32_t> ring_edge;

    bool build(int64_t n_vertices, int64_t n_faces, const int32_t* tri) {
        nv = n_vertices;
        // per lower endpoint: list of (upper endpoint, edge id); capacity from a count pass
        std::vector<int64_t> cap(n_vertices + 1, 0);
        for (int64_t f = 0; f < n_faces; f++) {
            const int32_t* t = tri + 3 * f;
            if (t[0] == t[1]) continue;
            for (int j = 0; j < 3; j++) {
                const int32_t a = t[j], b = t[(j + 1) % 3];
                if (a < 0 || b < 0 || a >= n_vertices || b >= n_vertices) return false;
                if (a == b) continue;
                cap[std::min(a, b) + 1]++;
            }
        }
        for (int64_t v = 0; v < n_vertices; v++) cap[v + 1] += cap[v];
        std::vector<int32_t> nb_up(cap[n_vertices]), nb_edge(cap[n_vertices]);
        std::vector<int32_t> fill(n_vertices, 0);
        v1.clear(); v2.clear(); poly1.clear(); poly2.clear(); extra_faces.clear();
        for (int64_t f = 0; f < n_faces; f++) {
            const int32_t* t = tri + 3 * f;
            if (t[0] == t[1]) continue;
            for (int j = 0; j < 3; j++) {
                const int32_t a = t[j], b = t[(j + 1) % 3];
                if (a == b) continue;
                const int32_t lo = std::min(a, b), hi = std::max(a, b);
                const int64_t base = cap[lo];
                int32_t e = -1;
                for (int32_t q = 0; q < fill[lo]; q++)
                    if (nb_up[base + q] == hi) { e = nb_edge[base + q]; break; }
                if (e >= 0) {
                    if (poly1[e] < 0) poly1[e] = (int32_t)f;
                    else if (poly2[e] >= 0) extra_faces.push_back({e, (int32_t)f});
                    else poly2[e] = (int32_t)f;
                    continue;
                }
                e = (int32_t)v1.size();
                v1.push_back(a); v2.push_back(b); poly1.push_back((int32_t)f); poly2.push_back(-1);
                nb_up[base + fill[lo]] = hi;
                nb_edge[base + fill[lo]] = e;
                fill[lo]++;
            }
        }
        // rings: edges in creation order (increasing id)
        ring_row.assign(n_vertices + 1, 0);
        const int64_t ne = (int64_t)v1.size();
        for (int64_t e = 0; e < ne; e++) { ring_row[v1[e] + 1]++; ring_row[v2[e] + 1]++; }
        for (int64_t v = 0; v < n_vertices; v++) ring_row[v + 1] += ring_row[v];
        ring_edge.resize(2 * ne);
        std::vector<int64_t> pos(ring_row.begin(), ring_row.end() - 1);
        for (int64_t e = 0; e < ne; e++) {
            ring_edge[pos[v1[e]]++] = (int32_t)e;
            ring_edge[pos[v2[e]]++] = (int32_t)e;
        }
        return true;
    }

    // vtkSurfaceBase::GetVertexNeighbourFaces (.cxx:964-984)
    void vertex_faces(int64_t v, std::vector<int32_t>& out) const {
        out.clear();
        auto ins = [&](int32_t f) {
            for (int32_t x : out) if (x == f) return;
            out.push_back(f);
        };
        for (int64_t p = ring_row[v]; p < ring_row[v + 1]; p++) {
            const int32_t e = ring_edge[p];
            if (poly1[e] >= 0) ins(poly1[e]);
            if (poly2[e] >= 0) ins(poly2[e]);
            if (!extra_faces.empty())
                for (auto& pr : extra_faces) if (pr.first == e) ins(pr.second);
        }
    }
};

double tri_area(const double* a, const double* b, const double* c) {
    auto d2 = [](const double* p, const double* q) {
        const double x = p[0] - q[0], y = p[1] - q[1], z = p[2] - q[2];
        return x * x + y * y + z * z;
    };
    const double A = d2(a, b), B = d2(b, c), C = d2(c, a);
    return 0.25 * std::sqrt(std::fabs(4.0 * A * C - (A - B + C) * (A - B + C)));
}

}  // namespace

extern "C" {

int acvd_build_topology(int64_t n_vertices, int64_t n_faces, const int32_t* tri, int32_t* csr_row,
                        int32_t* csr_col, int32_t* edge_v, int64_t* n_edges) {
    if (n_vertices <= 0 || n_faces < 0 || !tri || !n_edges) return ACVD_ERR_ARG;
    if (n_vertices >= (int64_t)1 << 31) return ACVD_ERR_UNSUPPORTED;
    EdgeTable t;
    if (!t.build(n_vertices, n_faces, tri)) return ACVD_ERR_ARG;
    const int64_t ne = (int64_t)t.v1.size();
    if (2 * ne >= (int64_t)1 << 31) return ACVD_ERR_UNSUPPORTED;
    *n_edges = ne;
    if (edge_v)
        for (int64_t e = 0; e < ne; e++) { edge_v[2 * e] = t.v1[e]; edge_v[2 * e + 1] = t.v2[e]; }
    if (csr_row && csr_col) {
        for (int64_t v = 0; v <= n_vertices; v++) csr_row[v] = (int32_t)t.ring_row[v];
        for (int64_t v = 0; v < n_vertices; v++)
            for (int64_t p = t.ring_row[v]; p < t.ring_row[v + 1]; p++) {
                const int32_t e = t.ring_edge[p];
                csr_col[p] = t.v1[e] == v ? t.v2[e] : t.v1[e];
            }
    }
    return ACVD_OK;
}

int acvd_vertex_weights(int metric, int64_t n_vertices, const double* xyz, int64_t n_faces, const int32_t* tri,
                        const int32_t* csr_row, const int32_t* csr_col, const int32_t* edge_v,
                        const double* indicator, double gradation, double* weights) {
    (void)csr_row; (void)csr_col; (void)edge_v;
    if (n_vertices <= 0 || !xyz || !tri || !weights) return ACVD_ERR_ARG;
    EdgeTable t;
    if (!t.build(n_vertices, n_faces, tri)) return ACVD_ERR_ARG;
    std::vector<double> farea(n_faces);
    for (int64_t f = 0; f < n_faces; f++)
        farea[f] = tri_area(xyz + 3 * tri[3 * f], xyz + 3 * tri[3 * f + 1], xyz + 3 * tri[3 * f + 2]);
    std::vector<int32_t> fl;
    const bool use_ind = indicator && (metric == ACVD_METRIC_QUADRIC_ANISOTROPIC ? gradation != 0.0 : gradation > 0.0);
    for (int64_t v = 0; v < n_vertices; v++) {
        t.vertex_faces(v, fl);
        double a = 0.0;
        for (int32_t f : fl) a += farea[f] / 3.0;
        double w = a;
        if (use_ind) w = a * std::pow(indicator[v], gradation);
        if (metric == ACVD_METRIC_QUADRIC_ANISOTROPIC) w = (double)(float)w;   // float item weights
        weights[v] = w;
    }
    const double ratio = metric == ACVD_METRIC_QEM ? 10000.0 : 100000.0;
    double avg = 0.0;
    for (int64_t v = 0; v < n_vertices; v++) avg += weights[v];
    avg /= (double)n_vertices;
    const double lo = avg / ratio, hi = avg * ratio;
    for (int64_t v = 0; v < n_vertices; v++) {
        double w = weights[v];
        if (w > hi) w = hi;
        if (w < lo) w = lo;
        if (metric == ACVD_METRIC_QUADRIC_ANISOTROPIC) w = (double)(float)w;
        weights[v] = w;
    }
    return ACVD_OK;
}

int acvd_initial_sampling(int64_t n_vertices, const int32_t* csr_row, const int32_t* csr_col,
                          const double* weights, int32_t k, int32_t* labels) {
    return acvd_initial_sampling_fixed(n_vertices, csr_row, csr_col, weights, k, 0, nullptr, labels);
}

int acvd_initial_sampling_fixed(int64_t n_vertices, const int32_t* csr_row, const int32_t* csr_col,
                                const double* weights, int32_t k, int32_t n_fixed, const int32_t* fixed_ids,
                                int32_t* labels) {
    if (n_vertices <= 0 || k <= 0 || !csr_row || !csr_col || !weights || !labels) return ACVD_ERR_ARG;
    if (n_fixed < 0 || n_fixed > k || (n_fixed > 0 && !fixed_ids)) return ACVD_ERR_ARG;
    const int64_t n = n_vertices;
    for (int64_t i = 0; i < n; i++) labels[i] = k;
    // the fixed vertices take clusters 0 .. F-1; the grown regions the labels above
    const int32_t offset = n_fixed;
    for (int32_t o = 0; o < offset; o++) {
        if (fixed_ids[o] < 0 || fixed_ids[o] >= n) return ACVD_ERR_ARG;
        labels[fixed_ids[o]] = o;
    }
    std::vector<int32_t> items(n);
    for (int64_t i = 0; i < n; i++) items[i] = (int32_t)i;
    std::mt19937 rng;
    rng.seed(0);
    for (int64_t i = n - 1; i > 0; --i) std::swap(items[i], items[rng() % (uint64_t)n]);
    double sw = 0.0;
    for (int64_t i = 0; i < n; i++) sw += weights[i];
    const double target = sw / (double)k;
    int64_t remaining_items = n;
    int32_t remaining = k - offset;
    int64_t first = 0;
    std::queue<int32_t> q;
    while (remaining_items > 0 && remaining > 0) {
        bool found = false;
        int32_t item = 0;
        while (!found && first < n) {
            item = items[first];
            if (labels[item] == k) found = true; else first++;
        }
        if (!found) break;
        while (!q.empty()) q.pop();
        q.push(item);
        sw = 0.0;
        remaining--;
        while (!q.empty()) {
            item = q.front();
            q.pop();
            if (labels[item] != k) continue;
            labels[item] = remaining + offset;
            sw += weights[item];
            remaining_items--;
            for (int32_t p = csr_row[item]; p < csr_row[item + 1]; p++) q.push(csr_col[p]);
            if (sw > target) break;
        }
    }
    if (remaining == 0) return ACVD_OK;
    // fewer grown regions than clusters: split single items off the larger ones
    std::vector<int32_t> sizes(k, 0);
    for (int64_t i = 0; i < n; i++) {
        items[i] = (int32_t)i;
        if (labels[i] != k) sizes[labels[i]]++;
    }
    for (int64_t i = n - 1; i > 0; --i) std::swap(items[i], items[rng() % (uint64_t)n]);
    first = 0;
    while (remaining) {
        int32_t item = 0;
        while (first < n) {
            item = items[first];
            first++;
            const int32_t cl = labels[item];
            if (cl == k) break;
            if (sizes[cl] == 1) continue;
            labels[item] = remaining + offset;
            sizes[cl]--;
            sizes[remaining + offset]++;
            break;
        }
        remaining--;
        labels[item] = remaining + offset;
    }
    return ACVD_OK;
}


// vtkSurface::SplitLongEdges (Common/vtkSurface.cxx:444-603) on the host.  The threshold
// is ratio x the mean edge length of the input; passes repeat until no edge is longer.
// A pass gives every edge longer than the threshold (and with a face) a midpoint vertex,
// appended in edge-id order and stored as float (vtkPoints), then splits each face with
// the reference's case table (Split2 / Split3 / four-way, :378-441, :524-582).  The
// reference's dynamic edge table decides the edge ids of later passes: a face's deletion
// frees, in the face's edge order, the edges left without a face into a FIFO that the
// next new edges draw from (vtkSurfaceBase.cxx:560-609, 1166-1221), and the first face
// of a split takes the deleted face's slot (:1223-1320).  That bookkeeping is simulated
// here, so vertices and faces come out in the reference's order.  The faces are taken
// as consistently oriented (the splits keep orientation; the reference's closing
// CheckNormals then changes nothing).
int acvd_split_long_edges(int64_t n_vertices, const double* xyz, int64_t n_faces, const int32_t* tri, double ratio,
                          double** out_xyz, int64_t* out_nv, int32_t** out_tri, int64_t* out_nf) {
    if (n_vertices <= 0 || n_faces < 0 || !xyz || (n_faces && !tri) || !out_xyz || !out_nv || !out_tri || !out_nf ||
        !(ratio > 0.0))
        return ACVD_ERR_ARG;
    *out_xyz = nullptr;
    *out_tri = nullptr;
    for (int64_t i = 0; i < 3 * n_faces; i++)
        if (tri[i] < 0 || tri[i] >= n_vertices) return ACVD_ERR_ARG;
    for (int64_t f = 0; f < n_faces; f++)
        if (tri[3 * f] == tri[3 * f + 1] || tri[3 * f + 1] == tri[3 * f + 2] || tri[3 * f] == tri[3 * f + 2])
            return ACVD_ERR_ARG;
    std::vector<double> pts(xyz, xyz + 3 * n_vertices);
    std::vector<int32_t> faces(tri, tri + 3 * n_faces);
    struct DynEdge {
        int32_t a, b;
        int nf;
        bool active;
    };
    std::vector<DynEdge> edges;
    std::unordered_map<uint64_t, int32_t> index;   // active edges by vertex pair
    std::queue<int32_t> freed;
    auto key = [](int32_t a, int32_t b) {
        const uint32_t lo = (uint32_t)std::min(a, b), hi = (uint32_t)std::max(a, b);
        return ((uint64_t)hi << 32) | lo;
    };
    auto add_edge = [&](int32_t a, int32_t b) {
        auto it = index.find(key(a, b));
        if (it != index.end()) {
            edges[it->second].nf++;
            return;
        }
        int32_t e;
        if (freed.empty()) {
            e = (int32_t)edges.size();
            edges.push_back({});
        } else {
            e = freed.front();
            freed.pop();
        }
        edges[e] = {a, b, 1, true};
        index[key(a, b)] = e;
    };
    auto add_face_edges = [&](const int32_t* f) {
        for (int j = 0; j < 3; j++) add_edge(f[j], f[(j + 1) % 3]);
    };
    auto delete_face_edges = [&](const int32_t* f) {
        for (int j = 0; j < 3; j++) {
            auto it = index.find(key(f[j], f[(j + 1) % 3]));
            DynEdge& e = edges[it->second];
            if (--e.nf == 0) {
                e.active = false;
                freed.push(it->second);
                index.erase(it);
            }
        }
    };
    auto edge_of = [&](int32_t a, int32_t b) { return index.at(key(a, b)); };
    for (int64_t f = 0; f < n_faces; f++) add_face_edges(&faces[3 * f]);
    auto length = [&](int32_t a, int32_t b) {
        const double dx = pts[3 * (size_t)a] - pts[3 * (size_t)b], dy = pts[3 * (size_t)a + 1] - pts[3 * (size_t)b + 1],
                     dz = pts[3 * (size_t)a + 2] - pts[3 * (size_t)b + 2];
        return std::sqrt(dx * dx + dy * dy + dz * dz);
    };
    double threshold = 0.0;
    for (const DynEdge& e : edges) threshold += length(e.a, e.b);
    threshold = edges.empty() ? 0.0 : ratio * threshold / (double)edges.size();
    for (bool split = !edges.empty(); split;) {
        split = false;
        std::vector<int32_t> mid(edges.size(), -1);
        for (size_t e = 0; e < edges.size(); e++) {
            if (!edges[e].active || length(edges[e].a, edges[e].b) <= threshold) continue;
            for (int c = 0; c < 3; c++)
                pts.push_back((double)(float)(0.5 * (pts[3 * (size_t)edges[e].a + c] + pts[3 * (size_t)edges[e].b + c])));
            mid[e] = (int32_t)(pts.size() / 3 - 1);
        }
        const size_t ncells = faces.size() / 3;
        for (size_t i = 0; i < ncells; i++) {
            const int32_t v1 = faces[3 * i], v2 = faces[3 * i + 1], v3 = faces[3 * i + 2];
            const int32_t v12 = mid[edge_of(v1, v2)], v13 = mid[edge_of(v1, v3)], v23 = mid[edge_of(v2, v3)];
            int32_t out[4][3];
            int n = 0;
            auto put = [&](int32_t a, int32_t b, int32_t c) {
                out[n][0] = a;
                out[n][1] = b;
                out[n][2] = c;
                n++;
            };
            // Split2(f, a, b, c, ab): (a, ab, c), (ab, b, c)
            auto split2 = [&](int32_t a, int32_t b, int32_t c, int32_t ab) {
                put(a, ab, c);
                put(ab, b, c);
            };
            // Split3(f, a, b, c, ab, ac): (a, ab, ac), (ab, b, c), (c, ac, ab)
            auto split3 = [&](int32_t a, int32_t b, int32_t c, int32_t ab, int32_t ac) {
                put(a, ab, ac);
                put(ab, b, c);
                put(c, ac, ab);
            };
            if (v12 < 0) {
                if (v13 < 0) {
                    if (v23 >= 0) split2(v2, v3, v1, v23);
                } else if (v23 < 0) {
                    split2(v3, v1, v2, v13);
                } else {
                    split3(v3, v1, v2, v13, v23);
                }
            } else if (v13 < 0) {
                if (v23 < 0) split2(v1, v2, v3, v12);
                else split3(v2, v3, v1, v23, v12);
            } else if (v23 < 0) {
                split3(v1, v2, v3, v12, v13);
            } else {
                put(v1, v12, v13);
                put(v12, v2, v23);
                put(v23, v3, v13);
                put(v12, v23, v13);
            }
            if (n == 0) continue;
            split = true;
            delete_face_edges(&faces[3 * i]);
            for (int k = 0; k < n; k++) {
                int32_t* dst;
                if (k == 0) {
                    dst = &faces[3 * i];   // the deleted face's slot
                } else {
                    faces.resize(faces.size() + 3);
                    dst = &faces[faces.size() - 3];
                }
                dst[0] = out[k][0];
                dst[1] = out[k][1];
                dst[2] = out[k][2];
                add_face_edges(dst);
            }
        }
        if (pts.size() / 3 > (size_t)INT32_MAX / 2) return ACVD_ERR_UNSUPPORTED;
    }
    *out_xyz = (double*)std::malloc(pts.size() * sizeof(double));
    *out_tri = (int32_t*)std::malloc(std::max<size_t>(faces.size(), 1) * sizeof(int32_t));
    if (!*out_xyz || !*out_tri) {
        std::free(*out_xyz);
        std::free(*out_tri);
        *out_xyz = nullptr;
        *out_tri = nullptr;
        return ACVD_ERR_ARG;
    }
    std::memcpy(*out_xyz, pts.data(), pts.size() * sizeof(double));
    std::memcpy(*out_tri, faces.data(), faces.size() * sizeof(int32_t));
    *out_nv = (int64_t)pts.size() / 3;
    *out_nf = (int64_t)faces.size() / 3;
    return ACVD_OK;
}

}  // extern "C"
