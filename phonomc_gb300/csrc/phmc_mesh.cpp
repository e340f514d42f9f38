// Surface-mesh geometry of mesh domains: readers, the closed-surface
// pipeline, the face BVH trace and the mesh form of SimulationDomain.
// Reference: src/geometry/MeshReader.cpp, src/SurfaceMesh.cpp,
// src/geometry/SurfaceSampling.cpp, src/SimulationDomain.cpp:73-126, 452-766.
#include "phmc_host.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstring>
#include <deque>
#include <fstream>
#include <functional>
#include <limits>
#include <map>
#include <numeric>
#include <queue>
#include <sstream>
#include <unordered_map>

namespace phmc {
namespace {
double dot3(const Vec3& a, const Vec3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
double norm3(const Vec3& a) { return std::sqrt(dot3(a, a)); }
Vec3 sub3(const Vec3& a, const Vec3& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }
Vec3 mul3(const Vec3& a, double s) { return {a[0] * s, a[1] * s, a[2] * s}; }
Vec3 add3(const Vec3& a, const Vec3& b) { return {a[0] + b[0], a[1] + b[1], a[2] + b[2]}; }
} // namespace

// ------------------------------------------------------ mesh tracing
namespace {
Vec3 vmin3(const Vec3& a, const Vec3& b) { return {std::min(a[0], b[0]), std::min(a[1], b[1]), std::min(a[2], b[2])}; }
Vec3 vmax3(const Vec3& a, const Vec3& b) { return {std::max(a[0], b[0]), std::max(a[1], b[1]), std::max(a[2], b[2])}; }
Vec3 cross3(const Vec3& a, const Vec3& b) {
    return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}

// src/SurfaceMesh.cpp:111-159: closest point of a triangle (Ericson's regions)
Vec3 closest_on_triangle(const Vec3& p, const Vec3& a, const Vec3& b, const Vec3& c) {
    const Vec3 ab = sub3(b, a), ac = sub3(c, a), ap = sub3(p, a);
    const double d1 = dot3(ab, ap), d2 = dot3(ac, ap);
    if (d1 <= 0.0 && d2 <= 0.0) return a;
    const Vec3 bp = sub3(p, b);
    const double d3 = dot3(ab, bp), d4 = dot3(ac, bp);
    if (d3 >= 0.0 && d4 <= d3) return b;
    const double vc = d1 * d4 - d3 * d2;
    if (vc <= 0.0 && d1 >= 0.0 && d3 <= 0.0) return add3(a, mul3(ab, d1 / (d1 - d3)));
    const Vec3 cp = sub3(p, c);
    const double d5 = dot3(ab, cp), d6 = dot3(ac, cp);
    if (d6 >= 0.0 && d5 <= d6) return c;
    const double vb = d5 * d2 - d1 * d6;
    if (vb <= 0.0 && d2 >= 0.0 && d6 <= 0.0) return add3(a, mul3(ac, d2 / (d2 - d6)));
    const double va = d3 * d6 - d5 * d4;
    if (va <= 0.0 && (d4 - d3) >= 0.0 && (d5 - d6) >= 0.0)
        return add3(b, mul3(sub3(c, b), (d4 - d3) / ((d4 - d3) + (d5 - d6))));
    const double denom = 1.0 / (va + vb + vc);
    return add3(add3(a, mul3(ab, vb * denom)), mul3(ac, vc * denom));
}

// src/SurfaceMesh.cpp:188-223
bool ray_box(const Vec3& o, const Vec3& d, const Vec3& bmin, const Vec3& bmax, double t_limit, double& t_near_out) {
    double t_near = 0.0, t_far = t_limit;
    for (int a = 0; a < 3; ++a) {
        if (std::abs(d[a]) <= 1e-14) {
            if (o[a] < bmin[a] - 1e-12 || o[a] > bmax[a] + 1e-12) return false;
            continue;
        }
        const double inv = 1.0 / d[a];
        double t0 = (bmin[a] - o[a]) * inv, t1 = (bmax[a] - o[a]) * inv;
        if (t0 > t1) std::swap(t0, t1);
        t_near = std::max(t_near, t0);
        t_far = std::min(t_far, t1);
        if (t_far < t_near) return false;
    }
    if (t_far <= 1e-10) return false;
    t_near_out = std::max(0.0, t_near);
    return t_near_out <= t_limit;
}
} // namespace

void MeshTracer::build(std::vector<Vec3> v, std::vector<std::array<int, 3>> f, std::vector<int> f2f) {
    vertices = std::move(v);
    faces = std::move(f);
    face_to_facet = std::move(f2f);
    const size_t nf = faces.size();
    if (face_to_facet.size() != nf) throw std::invalid_argument("face_to_facet must have one entry per face");
    normals.assign(nf, {0, 0, 0});
    centroids.assign(nf, {0, 0, 0});
    k.assign(nf, 0.0);
    bounds.assign(nf, {Vec3{0, 0, 0}, Vec3{0, 0, 0}});
    for (size_t i = 0; i < nf; ++i) {
        const Vec3 &a = vertices.at(faces[i][0]), &b = vertices.at(faces[i][1]), &c = vertices.at(faces[i][2]);
        const Vec3 n = cross3(sub3(b, a), sub3(c, a));
        const double area2 = norm3(n);
        normals[i] = area2 > 0.0 ? mul3(n, 1.0 / area2) : Vec3{0, 0, 0};
        centroids[i] = {(a[0] + b[0] + c[0]) / 3.0, (a[1] + b[1] + c[1]) / 3.0, (a[2] + b[2] + c[2]) / 3.0};
        k[i] = -dot3(normals[i], a);
        bounds[i] = {vmin3(vmin3(a, b), c), vmax3(vmax3(a, b), c)};
    }
    nodes.clear();
    order.clear();
    root = -1;
    if (nf <= 64) return; // a face scan is used below 65 faces
    order.resize(nf);
    std::iota(order.begin(), order.end(), 0);
    nodes.reserve(2 * nf);
    std::function<int(int, int)> split = [&](int begin, int end) -> int {
        const int id = static_cast<int>(nodes.size());
        nodes.push_back(Node{});
        Vec3 bmin = bounds[order[begin]][0], bmax = bounds[order[begin]][1];
        Vec3 cmin = centroids[order[begin]], cmax = cmin;
        for (int i = begin + 1; i < end; ++i) {
            bmin = vmin3(bmin, bounds[order[i]][0]);
            bmax = vmax3(bmax, bounds[order[i]][1]);
            cmin = vmin3(cmin, centroids[order[i]]);
            cmax = vmax3(cmax, centroids[order[i]]);
        }
        nodes[id].bmin = bmin;
        nodes[id].bmax = bmax;
        nodes[id].begin = begin;
        nodes[id].end = end;
        const int count = end - begin;
        if (count <= 8) return id;
        const Vec3 ext = sub3(cmax, cmin);
        int axis = 0;
        if (ext[1] > ext[axis]) axis = 1;
        if (ext[2] > ext[axis]) axis = 2;
        if (ext[axis] <= 1e-18) return id;
        const int mid = begin + count / 2;
        std::nth_element(order.begin() + begin, order.begin() + mid, order.begin() + end,
                         [&](int a, int b) { return centroids[a][axis] < centroids[b][axis]; });
        const int l = split(begin, mid);
        const int r = split(mid, end);
        nodes[id].left = l;
        nodes[id].right = r;
        return id;
    };
    root = split(0, static_cast<int>(nf));
}

void MeshTracer::trace(const Vec3& x, const Vec3& v, Vec3& hit, double& t_out, int& facet) const {
    double best_t = std::numeric_limits<double>::infinity();
    int best = -1;
    Vec3 best_p{0, 0, 0};
    auto try_face = [&](int i) {
        const double denom = dot3(v, normals[i]);
        if (std::abs(denom) < 1e-10) return;
        const double t = -(dot3(x, normals[i]) + k[i]) / denom;
        if (t <= 1e-10 || t >= best_t) return;
        const Vec3 p = add3(x, mul3(v, t));
        const auto& bb = bounds[i];
        if (p[0] < bb[0][0] - 1e-9 || p[1] < bb[0][1] - 1e-9 || p[2] < bb[0][2] - 1e-9 || p[0] > bb[1][0] + 1e-9 ||
            p[1] > bb[1][1] + 1e-9 || p[2] > bb[1][2] + 1e-9)
            return;
        const Vec3 cp = closest_on_triangle(p, vertices[faces[i][0]], vertices[faces[i][1]], vertices[faces[i][2]]);
        if (norm3(sub3(cp, p)) > 1e-7) return;
        best_t = t;
        best_p = p;
        best = i;
    };
    if (root >= 0) {
        int stack[64];
        int top = 0;
        stack[top++] = root;
        while (top > 0) {
            const Node& node = nodes[stack[--top]];
            double tn = 0.0;
            if (!ray_box(x, v, node.bmin, node.bmax, best_t, tn)) continue;
            if (node.left < 0 && node.right < 0) {
                for (int pos = node.begin; pos < node.end; ++pos) try_face(order[pos]);
                continue;
            }
            int near_child = -1, far_child = -1;
            double near_t = std::numeric_limits<double>::infinity(), far_t = near_t;
            for (int child : {node.left, node.right}) {
                if (child < 0) continue;
                double tc = 0.0;
                if (!ray_box(x, v, nodes[child].bmin, nodes[child].bmax, best_t, tc)) continue;
                if (tc < near_t) {
                    far_child = near_child;
                    far_t = near_t;
                    near_child = child;
                    near_t = tc;
                } else if (tc < far_t) {
                    far_child = child;
                    far_t = tc;
                }
            }
            if (far_child >= 0 && top < 64) stack[top++] = far_child;
            if (near_child >= 0 && top < 64) stack[top++] = near_child;
        }
    } else {
        for (size_t i = 0; i < faces.size(); ++i) try_face(static_cast<int>(i));
    }
    if (best < 0) {
        hit = x;
        t_out = std::numeric_limits<double>::infinity();
        facet = -1;
        return;
    }
    hit = best_p;
    t_out = best_t;
    facet = face_to_facet[best];
}


// ------------------------------------------------------------ readers
namespace {
std::string lower(std::string s) {
    for (char& c : s) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
    return s;
}

std::string extension(const std::string& path) {
    const size_t slash = path.find_last_of("/\\");
    const size_t dot = path.find_last_of('.');
    if (dot == std::string::npos || (slash != std::string::npos && dot < slash)) return "";
    return lower(path.substr(dot));
}

// Vertex merging on the lattice h = 1e-10 (src/geometry/MeshReader.cpp:41-63):
// equal rounded coordinates give the first vertex with that key.
struct VertexMerge {
    std::map<std::array<long long, 3>, int> index;
    std::vector<Vec3>& out;
    explicit VertexMerge(std::vector<Vec3>& v) : out(v) {}
    int add(const Vec3& p) {
        const std::array<long long, 3> key{std::llround(p[0] / 1e-10), std::llround(p[1] / 1e-10),
                                           std::llround(p[2] / 1e-10)};
        const auto it = index.find(key);
        if (it != index.end()) return it->second;
        const int id = static_cast<int>(out.size());
        out.push_back(p);
        index.emplace(key, id);
        return id;
    }
};

std::string trim(const std::string& s) {
    size_t b = 0, e = s.size();
    while (b < e && std::isspace(static_cast<unsigned char>(s[b]))) ++b;
    while (e > b && std::isspace(static_cast<unsigned char>(s[e - 1]))) --e;
    return s.substr(b, e - b);
}
} // namespace

void read_surface_mesh(const std::string& path, std::vector<Vec3>& vertices, std::vector<std::array<int, 3>>& faces) {
    vertices.clear();
    faces.clear();
    const std::string ext = extension(path);
    if (ext == ".obj") {
        std::ifstream in(path);
        if (!in) throw std::runtime_error("Failed to open OBJ file: " + path);
        std::string line;
        while (std::getline(in, line)) {
            const std::string t = trim(line);
            if (t.empty() || t[0] == '#') continue;
            std::istringstream iss(t);
            std::string tag;
            iss >> tag;
            if (tag == "v") {
                double x = 0, y = 0, z = 0;
                iss >> x >> y >> z;
                vertices.push_back({x, y, z});
            } else if (tag == "f") {
                std::vector<int> poly;
                std::string tok;
                while (iss >> tok) {
                    const std::string idx_s = tok.substr(0, tok.find('/'));
                    if (idx_s.empty()) continue;
                    int idx = std::stoi(idx_s);
                    idx = idx < 0 ? static_cast<int>(vertices.size()) + idx : idx - 1;
                    if (idx < 0 || idx >= static_cast<int>(vertices.size()))
                        throw std::runtime_error("OBJ face index out of range.");
                    poly.push_back(idx);
                }
                for (size_t i = 1; i + 1 < poly.size(); ++i) faces.push_back({poly[0], poly[i], poly[i + 1]});
            }
        }
        if (vertices.empty() || faces.empty()) throw std::runtime_error("OBJ mesh has no vertices/faces.");
        return;
    }
    if (ext != ".stl") throw std::runtime_error("Unsupported mesh extension: " + ext + " (expected .stl or .obj)");
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::runtime_error("Failed to open STL file: " + path);
    std::string bytes((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    // binary when the size matches the triangle count, or the file does not start with "solid"
    bool binary = false;
    if (bytes.size() >= 84) {
        uint32_t ntri = 0;
        std::memcpy(&ntri, bytes.data() + 80, 4);
        binary = 84ull + 50ull * ntri == bytes.size() || lower(bytes.substr(0, 5)) != "solid";
    }
    VertexMerge merge(vertices);
    if (binary) {
        uint32_t ntri = 0;
        std::memcpy(&ntri, bytes.data() + 80, 4);
        if (84ull + 50ull * ntri > bytes.size()) throw std::runtime_error("Truncated binary STL: " + path);
        for (uint32_t i = 0; i < ntri; ++i) {
            const char* rec = bytes.data() + 84 + 50ull * i + 12; // skip the stored normal
            int id[3];
            for (int k = 0; k < 3; ++k) {
                float c[3];
                std::memcpy(c, rec + 12 * k, 12);
                id[k] = merge.add({c[0], c[1], c[2]});
            }
            faces.push_back({id[0], id[1], id[2]});
        }
    } else {
        std::istringstream text(bytes);
        std::string line;
        std::vector<int> tri;
        while (std::getline(text, line)) {
            const std::string t = trim(line);
            if (t.size() < 6) continue;
            std::istringstream iss(t);
            std::string tag;
            iss >> tag;
            if (tag != "vertex") continue;
            double x = 0, y = 0, z = 0;
            iss >> x >> y >> z;
            tri.push_back(merge.add({x, y, z}));
            if (tri.size() == 3) {
                faces.push_back({tri[0], tri[1], tri[2]});
                tri.clear();
            }
        }
    }
    if (vertices.empty() || faces.empty()) throw std::runtime_error("STL mesh has no vertices/faces.");
}

// --------------------------------------------------------- surface mesh
namespace {
Vec3 normalize3(const Vec3& a) {
    const double n = norm3(a);
    if (n <= 0.0) return {0.0, 0.0, 0.0};
    return mul3(a, 1.0 / n);
}

// src/SurfaceMesh.cpp:71-101
std::array<std::array<double, 3>, 3> inverse3x3(const std::array<std::array<double, 3>, 3>& m, bool& ok) {
    const double a = m[0][0], b = m[0][1], c = m[0][2];
    const double d = m[1][0], e = m[1][1], f = m[1][2];
    const double g = m[2][0], h = m[2][1], i = m[2][2];
    const double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
    const double D = -(b * i - c * h), E = a * i - c * g, F = -(a * h - b * g);
    const double G = b * f - c * e, H = -(a * f - c * d), I = a * e - b * d;
    const double det = a * A + b * B + c * C;
    ok = !(std::abs(det) < 1e-14);
    if (!ok) return {};
    const double id = 1.0 / det;
    return {{{{A * id, D * id, G * id}}, {{B * id, E * id, H * id}}, {{C * id, F * id, I * id}}}};
}

// src/SurfaceMesh.cpp:162-186: Moller-Trumbore with eps 1e-10, hit when t > eps
bool ray_triangle(const Vec3& o, const Vec3& d, const Vec3& a, const Vec3& b, const Vec3& c, double& t) {
    constexpr double eps = 1e-10;
    const Vec3 e1 = sub3(b, a), e2 = sub3(c, a);
    const Vec3 pvec = cross3(d, e2);
    const double det = dot3(e1, pvec);
    if (std::abs(det) < eps) return false;
    const double inv_det = 1.0 / det;
    const Vec3 tvec = sub3(o, a);
    const double u = dot3(tvec, pvec) * inv_det;
    if (u < -eps || u > 1.0 + eps) return false;
    const Vec3 qvec = cross3(tvec, e1);
    const double v = dot3(d, qvec) * inv_det;
    if (v < -eps || (u + v) > 1.0 + eps) return false;
    t = dot3(e2, qvec) * inv_det;
    return t > eps;
}
} // namespace

void SurfaceMesh::set_data(std::vector<Vec3> vertices, std::vector<std::array<int, 3>> faces) {
    if (vertices.empty() || faces.empty()) throw std::runtime_error("SurfaceMesh requires non-empty vertices and faces.");
    for (const auto& f : faces)
        for (int k = 0; k < 3; ++k)
            if (f[k] < 0 || f[k] >= static_cast<int>(vertices.size()))
                throw std::runtime_error("Surface mesh face references a missing vertex.");
    vertices_ = std::move(vertices);
    faces_ = std::move(faces);
    rebuild();
}

// src/SurfaceMesh.cpp:254-261
void SurfaceMesh::shift_to_origin() {
    Vec3 lo = vertices_.front();
    for (const auto& v : vertices_) lo = vmin3(lo, v);
    for (auto& v : vertices_) v = sub3(v, lo);
    rebuild();
}

// src/SurfaceMesh.cpp:263-275
void SurfaceMesh::rebuild() {
    simplices_ready_ = false;
    simplices_.clear();
    bmin_ = vertices_.front();
    bmax_ = vertices_.front();
    for (const auto& v : vertices_) {
        bmin_ = vmin3(bmin_, v);
        bmax_ = vmax3(bmax_, v);
    }
    compute_edges();
    orient();
    compute_face_metrics();
    compute_facets();
    tracer_.build(vertices_, faces_, face_to_facet_);
    long double six = 0.0L; // :748-760
    for (const auto& f : faces_)
        six += static_cast<long double>(dot3(vertices_[f[0]], cross3(vertices_[f[1]], vertices_[f[2]])));
    volume_ = std::abs(static_cast<double>(six / 6.0L));
    if (!std::isfinite(volume_) || volume_ <= 1e-16)
        throw std::runtime_error("Surface mesh encloses no finite positive volume.");
}

// src/SurfaceMesh.cpp:431-453: edge ids in first-encounter order over the
// face pairs (0,1), (0,2), (1,2)
void SurfaceMesh::compute_edges() {
    std::unordered_map<unsigned long long, int> id;
    edges_.clear();
    edge_faces_.clear();
    face_edges_.assign(faces_.size(), {0, 0, 0});
    for (size_t face = 0; face < faces_.size(); ++face) {
        const auto& f = faces_[face];
        const std::array<std::array<int, 2>, 3> pairs{{{std::min(f[0], f[1]), std::max(f[0], f[1])},
                                                       {std::min(f[0], f[2]), std::max(f[0], f[2])},
                                                       {std::min(f[1], f[2]), std::max(f[1], f[2])}}};
        for (int j = 0; j < 3; ++j) {
            const unsigned long long key = (static_cast<unsigned long long>(pairs[j][0]) << 32) |
                                           static_cast<unsigned int>(pairs[j][1]);
            auto ins = id.emplace(key, static_cast<int>(edges_.size()));
            if (ins.second) {
                edges_.push_back(pairs[j]);
                edge_faces_.emplace_back();
            }
            face_edges_[face][j] = ins.first->second;
            edge_faces_[ins.first->second].push_back(static_cast<int>(face));
        }
    }
}

// src/SurfaceMesh.cpp:277-413
void SurfaceMesh::orient() {
    bool manifold = true;
    for (const auto& attached : edge_faces_) manifold = manifold && attached.size() == 2;
    if (!manifold) {
        // T-junctions: orient each face from the membership of points just off its centroid
        for (auto& f : faces_) {
            const Vec3 a = vertices_[f[0]], b = vertices_[f[1]], c = vertices_[f[2]];
            const Vec3 raw = cross3(sub3(b, a), sub3(c, a));
            const double length = norm3(raw);
            if (!(length > 0.0)) throw std::runtime_error("Degenerate triangle in CAD surface.");
            const Vec3 normal = mul3(raw, 1.0 / length);
            const Vec3 centroid = mul3(add3(add3(a, b), c), 1.0 / 3.0);
            const double edge = std::min({norm3(sub3(b, a)), norm3(sub3(c, a)), norm3(sub3(c, b))});
            bool resolved = false;
            for (double factor : {1e-8, 1e-7, 1e-6}) {
                const double eps = std::max(1e-8, edge * factor);
                const bool plus = contains_point_ray_cast(add3(centroid, mul3(normal, eps)));
                const bool minus = contains_point_ray_cast(add3(centroid, mul3(normal, -eps)));
                if (plus == minus) continue;
                if (plus) std::swap(f[1], f[2]);
                resolved = true;
                break;
            }
            if (!resolved)
                throw std::runtime_error("Cannot identify interior/exterior sides of CAD surface; check closure and "
                                         "overlapping faces.");
        }
        return;
    }
    auto direction = [&](int face, int u, int v) {
        const auto& f = faces_[face];
        for (int k = 0; k < 3; ++k) {
            const int a = f[k], b = f[(k + 1) % 3];
            if (a == u && b == v) return 1;
            if (a == v && b == u) return -1;
        }
        return 0;
    };
    std::vector<std::vector<std::array<int, 2>>> adjacency(faces_.size()); // (face, relation)
    for (size_t e = 0; e < edge_faces_.size(); ++e) {
        const int a = edge_faces_[e][0], b = edge_faces_[e][1];
        const int da = direction(a, edges_[e][0], edges_[e][1]);
        const int db = direction(b, edges_[e][0], edges_[e][1]);
        if (da == 0 || db == 0) throw std::runtime_error("Surface mesh edge-to-face topology is inconsistent.");
        const int relation = -da * db;
        adjacency[a].push_back({b, relation});
        adjacency[b].push_back({a, relation});
    }
    std::vector<int> orientation(faces_.size(), 0);
    std::vector<std::vector<int>> components;
    for (int root = 0; root < static_cast<int>(faces_.size()); ++root) {
        if (orientation[root] != 0) continue;
        components.emplace_back();
        std::queue<int> q;
        orientation[root] = 1;
        q.push(root);
        while (!q.empty()) {
            const int cur = q.front();
            q.pop();
            components.back().push_back(cur);
            for (const auto& c : adjacency[cur]) {
                const int required = orientation[cur] * c[1];
                int& assigned = orientation[c[0]];
                if (assigned == 0) {
                    assigned = required;
                    q.push(c[0]);
                } else if (assigned != required) {
                    throw std::runtime_error("Surface mesh is non-orientable or has inconsistent face winding.");
                }
            }
        }
    }
    for (const auto& comp : components) {
        long double six = 0.0L;
        for (int fi : comp) {
            const auto& f = faces_[fi];
            six += static_cast<long double>(orientation[fi]) *
                   static_cast<long double>(dot3(vertices_[f[0]], cross3(vertices_[f[1]], vertices_[f[2]])));
        }
        if (six < 0.0L)
            for (int fi : comp) orientation[fi] = -orientation[fi];
    }
    for (size_t i = 0; i < faces_.size(); ++i)
        if (orientation[i] < 0) std::swap(faces_[i][1], faces_[i][2]);
}

// src/SurfaceMesh.cpp:455-477
void SurfaceMesh::compute_face_metrics() {
    const size_t nf = faces_.size();
    face_normals_.assign(nf, {0, 0, 0});
    face_centroids_.assign(nf, {0, 0, 0});
    face_areas_.assign(nf, 0.0);
    for (size_t i = 0; i < nf; ++i) {
        const Vec3 &a = vertices_[faces_[i][0]], &b = vertices_[faces_[i][1]], &c = vertices_[faces_[i][2]];
        const Vec3 n = cross3(sub3(b, a), sub3(c, a));
        const double area2 = norm3(n);
        face_normals_[i] = area2 > 0.0 ? mul3(n, 1.0 / area2) : Vec3{0, 0, 0};
        face_areas_[i] = area2 * 0.5;
        face_centroids_[i] = {(a[0] + b[0] + c[0]) / 3.0, (a[1] + b[1] + c[1]) / 3.0, (a[2] + b[2] + c[2]) / 3.0};
    }
}

// src/SurfaceMesh.cpp:556-723: face adjacency, plane buckets, facets
void SurfaceMesh::compute_facets() {
    const int nf = static_cast<int>(faces_.size());
    face_adjacency_.clear();
    for (const auto& ef : edge_faces_)
        for (size_t i = 0; i < ef.size(); ++i)
            for (size_t j = i + 1; j < ef.size(); ++j)
                face_adjacency_.push_back({std::min(ef[i], ef[j]), std::max(ef[i], ef[j])});
    std::sort(face_adjacency_.begin(), face_adjacency_.end());
    face_adjacency_.erase(std::unique(face_adjacency_.begin(), face_adjacency_.end()), face_adjacency_.end());

    face_to_facet_.assign(nf, -1);
    facet_faces_.clear();
    facet_normals_.clear();
    facet_centroids_.clear();
    facet_areas_.clear();
    auto emit = [&](const std::vector<int>& members) {
        Vec3 nsum{0, 0, 0}, csum{0, 0, 0};
        double area = 0.0;
        for (int fi : members) {
            nsum = add3(nsum, face_normals_[fi]);
            csum = add3(csum, mul3(face_centroids_[fi], face_areas_[fi]));
            area += face_areas_[fi];
        }
        const int id = static_cast<int>(facet_faces_.size());
        for (int fi : members) face_to_facet_[fi] = id;
        facet_faces_.push_back(members);
        facet_normals_.push_back(normalize3(nsum));
        facet_areas_.push_back(area);
        facet_centroids_.push_back(area > 0.0 ? mul3(csum, 1.0 / area) : csum);
    };
    if (!merge_coplanar_) {
        for (int fi = 0; fi < nf; ++fi) emit({fi});
    } else {
        std::map<std::array<long long, 4>, int> bucket_of_key;
        std::vector<std::vector<int>> buckets;
        std::vector<int> bucket(nf);
        for (int i = 0; i < nf; ++i) {
            const Vec3& n = face_normals_[i];
            const double d = dot3(n, vertices_[faces_[i][0]]);
            const std::array<long long, 4> key{std::llround(n[0] * 1e6), std::llround(n[1] * 1e6),
                                               std::llround(n[2] * 1e6), std::llround(d * 1e6)};
            const auto ins = bucket_of_key.emplace(key, static_cast<int>(buckets.size()));
            if (ins.second) buckets.emplace_back();
            buckets[ins.first->second].push_back(i);
            bucket[i] = ins.first->second;
        }
        std::vector<std::vector<int>> neighbors(nf);
        for (const auto& adj : face_adjacency_) {
            neighbors[adj[0]].push_back(adj[1]);
            neighbors[adj[1]].push_back(adj[0]);
        }
        std::vector<char> visited(nf, 0);
        for (size_t b = 0; b < buckets.size(); ++b) {
            for (int seed : buckets[b]) {
                if (visited[seed]) continue;
                std::vector<int> component;
                std::queue<int> q;
                visited[seed] = 1;
                q.push(seed);
                while (!q.empty()) {
                    const int cur = q.front();
                    q.pop();
                    component.push_back(cur);
                    for (int nb : neighbors[cur]) {
                        if (visited[nb] || bucket[nb] != static_cast<int>(b)) continue;
                        visited[nb] = 1;
                        q.push(nb);
                    }
                }
                emit(component);
            }
        }
    }
    facet_boundary_edges_.assign(facet_faces_.size(), {});
    for (size_t f = 0; f < facet_faces_.size(); ++f) {
        std::map<int, int> count;
        for (int fi : facet_faces_[f])
            for (int e : face_edges_[fi]) count[e] += 1;
        for (const auto& [e, c] : count)
            if (c == 1) facet_boundary_edges_[f].push_back(e);
    }
}

std::vector<double> SurfaceMesh::facet_boundary_edge_lengths(int facet) const {
    std::vector<double> out;
    if (facet < 0 || facet >= facet_count()) return out;
    for (int e : facet_boundary_edges_[facet]) out.push_back(norm3(sub3(vertices_[edges_[e][0]], vertices_[edges_[e][1]])));
    std::sort(out.begin(), out.end());
    return out;
}

// src/SurfaceMesh.cpp:1100-1124
bool SurfaceMesh::contains_point_ray_cast(const Vec3& p) const {
    const Vec3 dir{1.0, 0.0, 0.0};
    std::vector<double> hits;
    for (const auto& f : faces_) {
        double t = 0.0;
        if (ray_triangle(p, dir, vertices_[f[0]], vertices_[f[1]], vertices_[f[2]], t)) hits.push_back(t);
    }
    if (hits.empty()) return false;
    std::sort(hits.begin(), hits.end());
    int unique = 1;
    for (size_t i = 1; i < hits.size(); ++i)
        if (std::abs(hits[i] - hits[i - 1]) > 1e-9) ++unique;
    return unique % 2 == 1;
}

// Star decomposition from the vertex mean (or the box centre when the mean is
// outside), discarded when its volume misses the enclosed volume by > 1e-3
// (src/SurfaceMesh.cpp:771-817, 931-936; the qdelaunay call fails without the
// external program and falls back to this).
void SurfaceMesh::build_simplices() const {
    simplices_.clear();
    Vec3 center{0, 0, 0};
    for (const auto& v : vertices_) center = add3(center, v);
    center = mul3(center, 1.0 / static_cast<double>(vertices_.size()));
    if (!contains_point_ray_cast(center)) center = mul3(add3(bmin_, bmax_), 0.5);
    for (const auto& f : faces_) {
        const Vec3 a = vertices_[f[0]], b = vertices_[f[1]], c = vertices_[f[2]];
        const double vol = std::abs(dot3(sub3(a, center), cross3(sub3(b, center), sub3(c, center)))) / 6.0;
        if (vol <= 1e-16) continue;
        Simplex s;
        s.v = {center, a, b, c};
        s.volume = vol;
        s.bounds = {vmin3(vmin3(center, a), vmin3(b, c)), vmax3(vmax3(center, a), vmax3(b, c))};
        const std::array<std::array<double, 3>, 3> A{{{{a[0] - center[0], b[0] - center[0], c[0] - center[0]}},
                                                      {{a[1] - center[1], b[1] - center[1], c[1] - center[1]}},
                                                      {{a[2] - center[2], b[2] - center[2], c[2] - center[2]}}}};
        bool ok = false;
        s.inv = inverse3x3(A, ok);
        if (!ok) continue;
        simplices_.push_back(s);
    }
    double total = 0.0;
    for (const auto& s : simplices_) total += s.volume;
    const double rel = std::abs(total - volume_) / std::max(volume_, 1e-18);
    if (!std::isfinite(rel) || rel > 1e-3) simplices_.clear();
    simplices_ready_ = true;
}

const std::vector<SurfaceMesh::Simplex>& SurfaceMesh::simplices() const {
    if (!simplices_ready_) build_simplices();
    return simplices_;
}

// src/SurfaceMesh.cpp:1126-1152
bool SurfaceMesh::contains_point(const Vec3& p) const {
    const auto& S = simplices();
    if (S.empty()) return contains_point_ray_cast(p);
    constexpr double tol = 1e-10;
    for (const auto& s : S) {
        if (p[0] < s.bounds[0][0] - tol || p[1] < s.bounds[0][1] - tol || p[2] < s.bounds[0][2] - tol ||
            p[0] > s.bounds[1][0] + tol || p[1] > s.bounds[1][1] + tol || p[2] > s.bounds[1][2] + tol)
            continue;
        const Vec3 d = sub3(p, s.v[0]);
        const double l1 = s.inv[0][0] * d[0] + s.inv[0][1] * d[1] + s.inv[0][2] * d[2];
        const double l2 = s.inv[1][0] * d[0] + s.inv[1][1] * d[1] + s.inv[1][2] * d[2];
        const double l3 = s.inv[2][0] * d[0] + s.inv[2][1] * d[1] + s.inv[2][2] * d[2];
        const double l0 = 1.0 - l1 - l2 - l3;
        if (l0 >= -tol && l1 >= -tol && l2 >= -tol && l3 >= -tol && l0 <= 1.0 + tol && l1 <= 1.0 + tol &&
            l2 <= 1.0 + tol && l3 <= 1.0 + tol)
            return true;
    }
    return contains_point_ray_cast(p);
}

// src/SurfaceMesh.cpp:996-1023: brute-force nearest face, first minimum
int SurfaceMesh::nearest_facet(const Vec3& p) const {
    int best = -1;
    double bd = std::numeric_limits<double>::infinity();
    for (size_t i = 0; i < faces_.size(); ++i) {
        const Vec3 cp = closest_on_triangle(p, vertices_[faces_[i][0]], vertices_[faces_[i][1]], vertices_[faces_[i][2]]);
        const double d = norm3(sub3(p, cp));
        if (d < bd) {
            bd = d;
            best = static_cast<int>(i);
        }
    }
    return best < 0 ? -1 : face_to_facet_[best];
}

// ------------------------------------------------------ mesh domain
// src/SimulationDomain.cpp:73-90 (construction order), 127-198 (mesh input),
// 452-516 (boundary regions), 518-624 (periodic pairs), 626-766 (cells).
void SimulationDomain::build_mesh_domain(const SimulationConfig& cfg) {
    std::vector<Vec3> verts;
    std::vector<std::array<int, 3>> faces;
    if (cfg.model == "mesh") {
        verts = cfg.mesh_vertices;
        faces = cfg.mesh_faces;
    } else {
        read_surface_mesh(cfg.model, verts, faces);
        if (extension(cfg.model) == ".stl") // STL lengths are nm; internal lengths are Angstrom
            for (auto& v : verts)
                for (double& x : v) x *= 10.0;
    }
    mesh_ = std::make_unique<SurfaceMesh>();
    mesh_->set_merge_coplanar_facets(cfg.merge_coplanar_facets);
    mesh_->set_data(std::move(verts), std::move(faces));
    mesh_->shift_to_origin();
    const SurfaceMesh& M = *mesh_;
    bmin_ = M.bounds_min();
    bmax_ = M.bounds_max();
    volume_ = M.volume();
    const int nf = M.facet_count();
    facets_.assign(nf, Facet{});
    for (int f = 0; f < nf; ++f) {
        Facet& F = facets_[f];
        F.normal = M.facet_normals()[f];
        F.centroid = M.facet_centroids()[f];
        F.area = M.facet_areas()[f];
        for (int fi : M.facet_faces()[f]) {
            const auto& t = M.faces()[fi];
            F.tris.push_back({M.vertices()[t[0]], M.vertices()[t[1]], M.vertices()[t[2]]});
            F.tri_area.push_back(M.face_areas()[fi]);
        }
    }

    // extruded prism: vertical sides, flat top and bottom; the top triangles
    // (src/SimulationDomain.cpp:206-231)
    prism_ = cfg.extruded_z;
    if (prism_) {
        const double tol = 1e-10 * std::max(1.0, bmax_[2] - bmin_[2]);
        double area = 0.0;
        for (const auto& f : M.faces()) {
            const std::array<Vec3, 3> tri{M.vertices()[f[0]], M.vertices()[f[1]], M.vertices()[f[2]]};
            bool top = true, bottom = true;
            for (const auto& q : tri) {
                top = top && std::abs(q[2] - bmax_[2]) < tol;
                bottom = bottom && std::abs(q[2] - bmin_[2]) < tol;
            }
            const double twice = (tri[1][0] - tri[0][0]) * (tri[2][1] - tri[0][1]) -
                                 (tri[1][1] - tri[0][1]) * (tri[2][0] - tri[0][0]);
            if (top) {
                prism_top_.push_back(tri);
                area += std::abs(twice) * 0.5;
            } else if (!bottom && std::abs(twice) > tol * tol) {
                throw std::runtime_error("extruded_z requires vertical sides and planar top/bottom");
            }
        }
        if (prism_top_.empty() || std::abs(area * (bmax_[2] - bmin_[2]) - volume_) > 1e-8 * volume_)
            throw std::runtime_error("extruded_z top area and mesh volume disagree");
    }

    const Vec3 ext = sub3(bmax_, bmin_);
    auto facets_in_region = [&](const std::array<double, 6>& box) {
        const double tolerance = 1e-12 * std::max({1.0, std::abs(ext[0]), std::abs(ext[1]), std::abs(ext[2])});
        Vec3 lo, hi;
        for (int a = 0; a < 3; ++a) {
            lo[a] = bmin_[a] + std::min(box[a], box[a + 3]) * ext[a];
            hi[a] = bmin_[a] + std::max(box[a], box[a + 3]) * ext[a];
        }
        std::vector<int> matched;
        for (int f = 0; f < nf; ++f) {
            const Vec3& c = facets_[f].centroid;
            bool inside = true;
            for (int a = 0; a < 3; ++a) inside = inside && c[a] >= lo[a] - tolerance && c[a] <= hi[a] + tolerance;
            if (inside) matched.push_back(f);
        }
        return matched;
    };

    // boundary conditions: unselected facets are smooth rough walls (eta = 0)
    const size_t nreg = cfg.boundary_position.size();
    if (cfg.boundary_conditions.size() != nreg || cfg.boundary_values.size() != nreg)
        throw std::runtime_error("boundary_position, boundary_conditions, and boundary_values must have identical "
                                 "lengths.");
    for (size_t i = 0; i < nreg; ++i) {
        const char cond = cfg.boundary_conditions[i];
        if (cond != 'T' && cond != 'P' && cond != 'R') throw std::runtime_error("Unknown boundary condition.");
        const double value = cond == 'R' ? cfg.boundary_values[i] * 10.0 : cfg.boundary_values[i];
        if (!std::isfinite(value) || value < 0 || (cond == 'P' && value != 0))
            throw std::runtime_error("Boundary values must be finite, nonnegative, and zero for periodic boundaries.");
        const auto matched = facets_in_region(cfg.boundary_position[i]);
        if (matched.empty())
            throw std::runtime_error("boundary_position region " + std::to_string(i) + " did not match any mesh facet.");
        for (int f : matched) {
            facets_[f].condition = cond;
            facets_[f].value = value;
        }
    }
    for (int f = 0; f < nf; ++f) {
        if (facets_[f].condition == 'T') {
            facets_[f].reservoir = static_cast<int>(reservoir_facets_.size());
            reservoir_facets_.push_back(f);
        }
    }

    // periodic pairs
    if (cfg.periodic_pair.size() % 2 != 0) throw std::runtime_error("periodic_pair must have even number of regions.");
    for (size_t i = 0; i < cfg.periodic_pair.size(); i += 2) {
        const auto A = facets_in_region(cfg.periodic_pair[i]);
        const auto B = facets_in_region(cfg.periodic_pair[i + 1]);
        if (A.empty() || B.empty()) throw std::runtime_error("Connected facet mapping failed for periodic_pair regions.");
        if (A.size() != B.size())
            throw std::runtime_error("periodic_pair region pair must match the same number of facets.");
        std::vector<std::array<int, 2>> pairs;
        if (A.size() == 1) {
            pairs.push_back({A[0], B[0]});
        } else {
            Vec3 ma{0, 0, 0}, mb{0, 0, 0};
            for (int fa : A) ma = add3(ma, facets_[fa].centroid);
            for (int fb : B) mb = add3(mb, facets_[fb].centroid);
            ma = mul3(ma, 1.0 / static_cast<double>(A.size()));
            mb = mul3(mb, 1.0 / static_cast<double>(B.size()));
            const Vec3 guess = sub3(mb, ma);
            std::vector<int> open = B;
            for (int fa : A) {
                const Vec3 target = add3(facets_[fa].centroid, guess);
                double best_d2 = std::numeric_limits<double>::infinity();
                int best = -1;
                for (int j = 0; j < static_cast<int>(open.size()); ++j) {
                    const Vec3 d = sub3(facets_[open[j]].centroid, target);
                    const double d2 = dot3(d, d);
                    if (d2 < best_d2) {
                        best_d2 = d2;
                        best = j;
                    }
                }
                if (best < 0) throw std::runtime_error("Failed to build one-to-one mapping for periodic_pair facets.");
                pairs.push_back({fa, open[best]});
                open.erase(open.begin() + best);
            }
        }
        for (const auto& pr : pairs) {
            Facet& a = facets_[pr[0]];
            Facet& b = facets_[pr[1]];
            if (a.condition != 'P' || b.condition != 'P')
                throw std::runtime_error("Connected facets must both be periodic ('P').");
            if ((a.pair >= 0 && a.pair != pr[1]) || (b.pair >= 0 && b.pair != pr[0]))
                throw std::runtime_error("Facet already paired with a different periodic connection.");
            if (dot3(a.normal, b.normal) > -0.98)
                throw std::runtime_error("Connected facets normals do not match opposite direction.");
            if (std::abs(a.area - b.area) / std::max({1.0, a.area, b.area}) > 1e-3)
                throw std::runtime_error("Connected facets area mismatch.");
            const auto la = M.facet_boundary_edge_lengths(pr[0]);
            const auto lb = M.facet_boundary_edge_lengths(pr[1]);
            if (la.size() != lb.size()) throw std::runtime_error("Connected facets boundary edge count mismatch.");
            for (size_t k = 0; k < la.size(); ++k)
                if (std::abs(la[k] - lb[k]) / std::max({1.0, la[k], lb[k]}) > 1e-3)
                    throw std::runtime_error("Connected facets boundary edge-length spectrum mismatch.");
            a.pair = pr[1];
            b.pair = pr[0];
            a.shift = sub3(b.centroid, a.centroid);
            b.shift = sub3(a.centroid, b.centroid);
        }
    }
    for (int f = 0; f < nf; ++f)
        if (facets_[f].condition == 'P' && facets_[f].pair < 0)
            throw std::runtime_error("Periodic boundary facet " + std::to_string(f) + " is not assigned to a periodic pair.");

    // cells: voxel centres inside the mesh, the rest mapped by a six-neighbour BFS
    const int nx = cfg.grid[0], ny = cfg.grid[1], nz = cfg.grid[2];
    if (nx <= 0 || ny <= 0 || nz <= 0) throw std::runtime_error("Grid sizes must be positive.");
    shape_ = {nx, ny, nz};
    inv_cell_ = {ext[0] > 0.0 ? nx / ext[0] : 0.0, ext[1] > 0.0 ? ny / ext[1] : 0.0, ext[2] > 0.0 ? nz / ext[2] : 0.0};
    const size_t total = static_cast<size_t>(nx) * ny * nz;
    voxel_cell_.assign(total, -1);
    auto voxel_centre = [&](size_t v) {
        const int ix = static_cast<int>(v / (static_cast<size_t>(ny) * nz)), iy = static_cast<int>(v / nz % ny),
                  iz = static_cast<int>(v % nz);
        return Vec3{bmin_[0] + (ix + 0.5) * ext[0] / nx, bmin_[1] + (iy + 0.5) * ext[1] / ny,
                    bmin_[2] + (iz + 0.5) * ext[2] / nz};
    };
    if (prism_) {
        build_prism_cells(nx, ny, nz);
    } else {
        // membership in parallel (the lazily built decomposition first), cell
        // numbers in voxel order
        (void)M.simplices();
        std::vector<unsigned char> inside(total, 0);
#pragma omp parallel for schedule(dynamic, 256)
        for (long long v = 0; v < static_cast<long long>(total); ++v)
            inside[v] = M.contains_point(voxel_centre(static_cast<size_t>(v))) ? 1 : 0;
        for (size_t v = 0; v < total; ++v) {
            if (!inside[v]) continue;
            voxel_cell_[v] = static_cast<int>(centers_.size());
            centers_.push_back(voxel_centre(v));
        }
        // interior voxels: the closed surface does not cross a box that no
        // face's bounding box reaches, so the whole box shares its centre's side
        const double margin = 1e-6 * std::max({1.0, ext[0], ext[1], ext[2]});
        std::vector<unsigned char> touched(total, 0);
        const auto& V = M.vertices();
        for (const auto& fc : M.faces()) {
            int lo[3], hi[3];
            for (int a = 0; a < 3; ++a) {
                const double fmin = std::min({V[fc[0]][a], V[fc[1]][a], V[fc[2]][a]}) - margin;
                const double fmax = std::max({V[fc[0]][a], V[fc[1]][a], V[fc[2]][a]}) + margin;
                const int n = shape_[a];
                // the margin (1e-6 of the scale) dwarfs the rounding of these indices
                lo[a] = std::max(0, static_cast<int>(std::floor((fmin - bmin_[a]) * inv_cell_[a])));
                hi[a] = std::min(n - 1, static_cast<int>(std::floor((fmax - bmin_[a]) * inv_cell_[a])));
            }
            for (int ix = lo[0]; ix <= hi[0]; ++ix)
                for (int iy = lo[1]; iy <= hi[1]; ++iy)
                    for (int iz = lo[2]; iz <= hi[2]; ++iz) touched[(static_cast<size_t>(ix) * ny + iy) * nz + iz] = 1;
        }
        voxel_interior_.assign(total, 0);
        for (size_t v = 0; v < total; ++v) voxel_interior_[v] = inside[v] && !touched[v] ? 1 : 0;
    }
    if (centers_.empty()) throw std::runtime_error("No valid grid centers found inside mesh.");
    std::deque<int> queue;
    for (size_t c = 0; c < total; ++c)
        if (voxel_cell_[c] >= 0) queue.push_back(static_cast<int>(c));
    const int yz = ny * nz;
    while (!queue.empty()) {
        const int c = queue.front();
        queue.pop_front();
        const int ix = c / yz, iy = (c % yz) / nz, iz = (c % yz) % nz;
        const int src = voxel_cell_[c];
        const int nb[6][3] = {{ix - 1, iy, iz}, {ix + 1, iy, iz}, {ix, iy - 1, iz},
                              {ix, iy + 1, iz}, {ix, iy, iz - 1}, {ix, iy, iz + 1}};
        for (const auto& n : nb) {
            if (n[0] < 0 || n[0] >= nx || n[1] < 0 || n[1] >= ny || n[2] < 0 || n[2] >= nz) continue;
            const int next = (n[0] * ny + n[1]) * nz + n[2];
            if (voxel_cell_[next] >= 0) continue;
            voxel_cell_[next] = src;
            queue.push_back(next);
        }
    }
    if (!prism_) {
        volumes_.assign(centers_.size(), volume_ / static_cast<double>(centers_.size()));
    } else {
        long double sum = 0;
        for (double v : volumes_) sum += v;
        if (std::abs(sum - volume_) > 1e-8 * volume_) throw std::runtime_error("Prism cut-cell volumes do not close");
    }
}

// Cells of an extruded prism (src/SimulationDomain.cpp:650-711): per voxel
// column the top triangles clipped to the column (Sutherland-Hodgman over its
// four sides), areas and centroids of the clipped polygons summed in long
// double; a voxel is a cell when its cut volume exceeds 1e-12 of an average
// voxel's, at the area centroid in x and y and the voxel centre in z. The
// column's polygons do not depend on z, so they are clipped once per column.
void SimulationDomain::build_prism_cells(int nx, int ny, int nz) {
    const Vec3 ext = sub3(bmax_, bmin_);
    const size_t total = static_cast<size_t>(nx) * ny * nz;
    volumes_.clear();
    for (int ix = 0; ix < nx; ++ix)
        for (int iy = 0; iy < ny; ++iy) {
            const double x0 = bmin_[0] + ix * ext[0] / nx, x1 = x0 + ext[0] / nx;
            const double y0 = bmin_[1] + iy * ext[1] / ny, y1 = y0 + ext[1] / ny;
            long double area_sum = 0, cx = 0, cy = 0;
            for (const auto& tri : prism_top_) {
                std::vector<Vec3> poly(tri.begin(), tri.end());
                for (int edge = 0; edge < 4; ++edge) {
                    const int axis = edge / 2;
                    const bool lower = edge % 2 == 0;
                    const double bound = axis == 0 ? (lower ? x0 : x1) : (lower ? y0 : y1);
                    std::vector<Vec3> clipped;
                    for (size_t i = 0; i < poly.size(); ++i) {
                        const Vec3& a = poly[i];
                        const Vec3& b = poly[(i + 1) % poly.size()];
                        const bool ina = lower ? a[axis] >= bound : a[axis] <= bound;
                        const bool inb = lower ? b[axis] >= bound : b[axis] <= bound;
                        if (ina) clipped.push_back(a);
                        if (ina != inb) {
                            const double f = (bound - a[axis]) / (b[axis] - a[axis]);
                            clipped.push_back(add3(a, mul3(sub3(b, a), f)));
                        }
                    }
                    poly = std::move(clipped);
                }
                for (size_t i = 1; i + 1 < poly.size(); ++i) {
                    const Vec3& a = poly[0];
                    const Vec3& b = poly[i];
                    const Vec3& c = poly[i + 1];
                    const long double area =
                        std::abs((b[0] - a[0]) * (c[1] - a[1]) - (b[1] - a[1]) * (c[0] - a[0])) * .5;
                    area_sum += area;
                    cx += area * (a[0] + b[0] + c[0]) / 3;
                    cy += area * (a[1] + b[1] + c[1]) / 3;
                }
            }
            const double cut_volume = static_cast<double>(area_sum) * ext[2] / nz;
            for (int iz = 0; iz < nz; ++iz) {
                Vec3 q{bmin_[0] + (static_cast<double>(ix) + 0.5) * ext[0] / static_cast<double>(nx),
                       bmin_[1] + (static_cast<double>(iy) + 0.5) * ext[1] / static_cast<double>(ny),
                       bmin_[2] + (static_cast<double>(iz) + 0.5) * ext[2] / static_cast<double>(nz)};
                if (area_sum > 0) {
                    q[0] = static_cast<double>(cx / area_sum);
                    q[1] = static_cast<double>(cy / area_sum);
                }
                if (cut_volume > 1e-12 * volume_ / static_cast<double>(total)) {
                    voxel_cell_[(static_cast<size_t>(ix) * ny + iy) * nz + iz] = static_cast<int>(centers_.size());
                    centers_.push_back(q);
                    volumes_.push_back(cut_volume);
                }
            }
        }
}

// Trace of an extruded prism (src/SimulationDomain.cpp:344-396): every facet's
// plane through its centroid, the nearest positive distance along the unit
// direction, the hit kept when it lies in one of the facet's triangles by
// long-double edge functions in the projection that drops the normal's
// largest axis (tolerance 1e-12 of the triangle's projected area).
void SimulationDomain::prism_trace(const Vec3& position, const Vec3& velocity, Vec3& cp, double& t,
                                   int& facet) const {
    const double speed = norm3(velocity);
    cp = position;
    t = std::numeric_limits<double>::infinity();
    facet = -1;
    if (!(speed > 0)) return;
    const Vec3 direction = mul3(velocity, 1 / speed);
    const SurfaceMesh& M = *mesh_;
    double best = std::numeric_limits<double>::infinity();
    for (int f = 0; f < M.facet_count(); ++f) {
        const Vec3& n = M.facet_normals()[f];
        const double denominator = dot3(direction, n);
        if (denominator <= 1e-16) continue;
        const double distance = dot3(sub3(M.facet_centroids()[f], position), n) / denominator;
        if (distance <= 1e-12 || distance >= best) continue;
        const Vec3 candidate = add3(position, mul3(direction, distance));
        int drop = 0;
        for (int j = 1; j < 3; ++j)
            if (std::abs(n[j]) > std::abs(n[drop])) drop = j;
        const int u = (drop + 1) % 3, v = (drop + 2) % 3;
        auto cross2 = [&](const Vec3& a, const Vec3& b, const Vec3& c) {
            return (static_cast<long double>(b[u]) - a[u]) * (static_cast<long double>(c[v]) - a[v]) -
                   (static_cast<long double>(b[v]) - a[v]) * (static_cast<long double>(c[u]) - a[u]);
        };
        for (int face : M.facet_faces()[f]) {
            const auto& id = M.faces()[face];
            const Vec3& a = M.vertices()[id[0]];
            const Vec3& b = M.vertices()[id[1]];
            const Vec3& c = M.vertices()[id[2]];
            const long double area = cross2(a, b, c), tol = 1e-12L * std::abs(area);
            const long double e0 = cross2(a, b, candidate), e1 = cross2(b, c, candidate), e2 = cross2(c, a, candidate);
            if ((area > 0 && std::min({e0, e1, e2}) >= -tol) || (area < 0 && std::max({e0, e1, e2}) <= tol)) {
                best = distance;
                facet = f;
                cp = candidate;
                break;
            }
        }
    }
    t = best / speed;
}

} // namespace phmc
