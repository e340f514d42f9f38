// Acoustic-mismatch interface tables: the reference's AcousticInterfaceSampler
// (src/solver/AcousticInterfaceSampler.cpp:18-472) with the channel-cell
// geometry it uses (src/solver/ChannelCell.cpp:1-210), restated step for step
// so the transmitted rows -- and therefore the sampled outgoing modes -- are
// the reference's. Built once on the host; the device samples the rows.
#include "phmc_host.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <map>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <string>
#include <tuple>
#include <unordered_map>

namespace phmc {
namespace channel {
namespace {
using V = std::array<double, 3>;
using M = std::array<V, 3>;
using Face = std::vector<V>;
using Poly = std::vector<Face>;

V sub(V a, const V& b) {
    for (int j = 0; j < 3; ++j) a[j] -= b[j];
    return a;
}
double dot(const V& a, const V& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
V cross(const V& a, const V& b) {
    return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}
V mean(const Face& f) {
    V c{};
    for (const V& p : f)
        for (int j = 0; j < 3; ++j) c[j] += p[j] / f.size();
    return c;
}
bool close(const V& a, const V& b) {
    const V d = sub(a, b);
    return dot(d, d) < 1e-24;
}
void append(Face& f, const V& p) {
    if (f.empty() || !close(f.back(), p)) f.push_back(p);
}

// Keeps the part of a convex polyhedron with sign * n.(p - o) <= 1/2 (one
// face pair of a cell in its own coordinates); the cut becomes a new face
// whose vertices are ordered by angle around its mean.
Poly clip(const Poly& poly, const V& n, const V& o, double sign) {
    Poly result;
    Face cap;
    auto distance = [&](const V& p) { return sign * dot(n, sub(p, o)) - .5; };
    for (const Face& face : poly) {
        Face out;
        for (size_t i = 0; i < face.size(); ++i) {
            const V& a = face[i];
            const V& b = face[(i + 1) % face.size()];
            const double da = distance(a), db = distance(b);
            const bool ia = da <= 1e-12, ib = db <= 1e-12;
            if (ia) append(out, a);
            if (ia != ib) {
                const double t = da / (da - db);
                V x{};
                for (int j = 0; j < 3; ++j) x[j] = a[j] + t * (b[j] - a[j]);
                append(out, x);
                if (std::none_of(cap.begin(), cap.end(), [&](const V& c) { return close(c, x); })) cap.push_back(x);
            }
        }
        if (out.size() > 1 && close(out.front(), out.back())) out.pop_back();
        if (out.size() >= 3) result.push_back(std::move(out));
    }
    if (cap.size() >= 3) {
        const V c = mean(cap);
        V u0 = n;
        double norm = std::sqrt(dot(u0, u0));
        for (double& x : u0) x /= norm;
        V u = cross(u0, std::abs(u0[0]) < .8 ? V{1, 0, 0} : V{0, 1, 0});
        norm = std::sqrt(dot(u, u));
        for (double& x : u) x /= norm;
        const V w = cross(u0, u);
        std::sort(cap.begin(), cap.end(), [&](V a, V b) {
            a = sub(a, c);
            b = sub(b, c);
            return std::atan2(dot(a, w), dot(a, u)) < std::atan2(dot(b, w), dot(b, u));
        });
        result.push_back(std::move(cap));
    }
    return result;
}
} // namespace

// A parallelepiped of channel space: centre, full-width basis (columns are the
// edge vectors), its inverse rows and axis-aligned bounds.
struct Cell {
    V center{}, lower{}, upper{};
    M basis{}, inverse{};
    double volume = 0;
    Cell(V origin, M b) : center(origin), basis(b) {
        const V c0{b[0][0], b[1][0], b[2][0]}, c1{b[0][1], b[1][1], b[2][1]}, c2{b[0][2], b[1][2], b[2][2]};
        const double det = dot(c0, cross(c1, c2));
        volume = std::abs(det);
        if (!std::isfinite(volume) || volume <= 0) throw std::invalid_argument("Degenerate phonon channel cell");
        inverse = {cross(c1, c2), cross(c2, c0), cross(c0, c1)};
        for (V& row : inverse)
            for (double& x : row) x /= det;
        for (int i = 0; i < 3; ++i) {
            double radius = 0;
            for (int j = 0; j < 3; ++j) radius += .5 * std::abs(b[i][j]);
            lower[i] = center[i] - radius;
            upper[i] = center[i] + radius;
        }
    }
    V coordinates(const V& p) const {
        V y{};
        const V d = sub(p, center);
        for (int i = 0; i < 3; ++i) y[i] = dot(inverse[i], d);
        return y;
    }
    Poly polyhedron() const {
        std::array<V, 8> vx;
        for (int i = 0; i < 8; ++i) {
            vx[i] = center;
            for (int d = 0; d < 3; ++d)
                for (int j = 0; j < 3; ++j) vx[i][d] += basis[d][j] * ((i & (1 << j)) ? .5 : -.5);
        }
        static constexpr int faces[6][4] = {{0, 2, 6, 4}, {1, 3, 7, 5}, {0, 1, 5, 4},
                                            {2, 3, 7, 6}, {0, 1, 3, 2}, {4, 5, 7, 6}};
        Poly poly;
        for (const auto& f : faces) {
            Face face;
            for (int i : f) face.push_back(vx[i]);
            poly.push_back(std::move(face));
        }
        return poly;
    }
};

Poly intersect(const Cell& a, const Cell& b) {
    for (int i = 0; i < 3; ++i)
        if (a.upper[i] <= b.lower[i] || b.upper[i] <= a.lower[i]) return {};
    Poly poly = a.polyhedron();
    for (int i = 0; i < 3 && !poly.empty(); ++i)
        for (double s : {-1., 1.}) poly = clip(poly, b.inverse[i], b.center, s);
    return poly;
}

struct QPoint {
    V point;
    double weight;
};

// Tetrahedra from the vertex mean to every face fan, each with the symmetric
// four-point degree-two rule (barycentric weights (5 + 3 sqrt 5) / 20 and
// (5 - sqrt 5) / 20, a quarter of the volume per point).
std::vector<QPoint> quadrature(const Poly& poly) {
    Face all;
    for (const Face& f : poly)
        for (const V& x : f) all.push_back(x);
    if (all.empty()) return {};
    const V anchor = mean(all);
    std::vector<QPoint> pts;
    const double large = (5.0 + 3.0 * std::sqrt(5.0)) / 20.0, small = (5.0 - std::sqrt(5.0)) / 20.0;
    for (const Face& face : poly) {
        for (size_t i = 1; i + 1 < face.size(); ++i) {
            const std::array<V, 4> p{anchor, face[0], face[i], face[i + 1]};
            const double vol = std::abs(dot(sub(p[1], p[0]), cross(sub(p[2], p[0]), sub(p[3], p[0])))) / 6;
            if (vol <= 0) continue;
            for (int a = 0; a < 4; ++a) {
                V x{};
                for (int b = 0; b < 4; ++b)
                    for (int j = 0; j < 3; ++j) x[j] += (a == b ? large : small) * p[b][j];
                pts.push_back({x, vol / 4});
            }
        }
    }
    return pts;
}
} // namespace channel

double AmmTables::transmission(double z1, double z2, double c1, double c2) {
    if (!std::isfinite(z1) || !std::isfinite(z2) || !std::isfinite(c1) || !std::isfinite(c2) || z1 <= 0 || z2 <= 0 ||
        c1 < 0 || c2 < 0 || c1 > 1 || c2 > 1)
        throw std::invalid_argument("Invalid scalar acoustic impedance/angle.");
    const double a = z1 * c1, b = z2 * c2;
    return a + b > 0 ? std::clamp(4 * a * b / ((a + b) * (a + b)), 0.0, 1.0) : 0;
}

void AmmTables::build(const std::vector<const PhononMaterial*>& mats, int axis, const std::vector<double>& densities,
                      double df, double dk) {
    if (axis < 0 || axis > 2 || mats.size() < 2 || densities.size() != mats.size() || !std::isfinite(df) || df <= 0 ||
        !std::isfinite(dk) || dk <= 0)
        throw std::invalid_argument("AMM needs layered materials, mass densities and positive frequency/k-parallel bins.");
    const double pi = std::acos(-1.0);
    const int ta = (axis + 1) % 3, tb = (axis + 2) % 3;
    struct Mode {
        double omega, flux;
        Vec3 k, v;
        int branch;
    };
    const size_t nm = mats.size();
    std::vector<std::vector<Mode>> modes(nm);
    std::vector<std::vector<int>> mirror(nm);
    // 1. reflection partners: the mode at the mirrored reciprocal-grid address
    //    with equal frequency and mirrored velocity
    for (size_t m = 0; m < nm; ++m) {
        if (!mats[m] || !std::isfinite(densities[m]) || densities[m] <= 0)
            throw std::invalid_argument("AMM needs finite positive material densities.");
        const PhononMaterial& mat = *mats[m];
        const auto& mesh = mat.q_mesh();
        if (mesh[0] <= 0 || mesh[1] <= 0 || mesh[2] <= 0) throw std::runtime_error("AMM needs a complete uniform q mesh.");
        const channel::Cell reciprocal({0, 0, 0}, mat.reciprocal_lattice());
        using Key = std::array<long long, 3>;
        auto grid_key = [&](const Vec3& k) {
            const auto q = reciprocal.coordinates(k);
            Key key{};
            for (int j = 0; j < 3; ++j) {
                const double x = q[j] * 2 * mesh[j];
                const long long index = std::llround(x), period = 2LL * mesh[j];
                if (std::abs(x - index) > 1e-5)
                    throw std::runtime_error("Interface reflection does not preserve the material q grid.");
                key[j] = (index % period + period) % period;
            }
            return key;
        };
        const int n = mat.active_mode_count();
        const int nb = mat.branch_count();
        mirror[m].assign(n, -1);
        std::map<Key, int> qpoints;
        for (int i = 0; i < n; ++i) {
            const int flat = mat.active_flat()[i];
            const Vec3& v = mat.velocity(flat);
            modes[m].push_back({mat.omega(flat), std::abs(v[axis]) / mat.energy_density_normalization(),
                                mat.wavevector(flat), v, flat % nb});
            qpoints[grid_key(mat.wavevector(flat))] = flat / nb;
        }
        std::vector<int> optical_negative;
        for (int j = 0; j < n; ++j)
            if (modes[m][j].branch >= 3 && modes[m][j].v[axis] < -1e-7) optical_negative.push_back(j);
        std::sort(optical_negative.begin(), optical_negative.end(), [&](int i, int j) {
            return std::tie(modes[m][i].omega, i) < std::tie(modes[m][j].omega, j);
        });
        auto mismatch = [&](const Mode& x, const Mode& y) {
            double dv = 0, scale = 0;
            for (int d = 0; d < 3; ++d) {
                dv += std::pow(x.v[d] - (d == axis ? -y.v[d] : y.v[d]), 2);
                scale += x.v[d] * x.v[d];
            }
            return std::make_pair(dv, scale);
        };
        for (int i = 0; i < n; ++i) {
            const Mode& x = modes[m][i];
            if (x.v[axis] <= 1e-7) continue;
            Vec3 rk = x.k;
            rk[axis] *= -1;
            auto it = qpoints.find(grid_key(rk));
            if (it == qpoints.end()) throw std::runtime_error("AMM reflection has no reciprocal-grid partner.");
            int best = -1;
            double error = std::numeric_limits<double>::infinity();
            for (int branch = 0; branch < nb; ++branch) {
                if ((x.branch < 3) != (branch < 3)) continue;
                const int j = mat.active_index_for_flat(it->second * nb + branch);
                if (j < 0 || mirror[m][j] >= 0) continue;
                const Mode& y = modes[m][j];
                if (y.v[axis] >= -1e-7) continue;
                if (std::abs(x.omega - y.omega) > 1e-6 * std::max(x.omega, y.omega)) continue;
                auto [dv, scale] = mismatch(x, y);
                if (dv > 1e-12 * std::max(1., scale)) continue;
                dv += branch == x.branch ? 0 : 1e-24; // the original branch wins a degenerate tie
                if (dv < error) {
                    error = dv;
                    best = j;
                }
            }
            if (best < 0 && x.branch >= 3) { // an optical mirror elsewhere in the branch
                const double tol = 1e-6 * x.omega;
                auto first = std::lower_bound(optical_negative.begin(), optical_negative.end(), x.omega - tol,
                                              [&](int j, double w) { return modes[m][j].omega < w; });
                for (auto jt = first; jt != optical_negative.end() && modes[m][*jt].omega <= x.omega + tol; ++jt) {
                    const int j = *jt;
                    const Mode& y = modes[m][j];
                    if (mirror[m][j] >= 0 || y.branch != x.branch) continue;
                    const auto [dv, scale] = mismatch(x, y);
                    if (dv <= 1e-12 * std::max(1., scale) && dv < error) {
                        error = dv;
                        best = j;
                    }
                }
            }
            if (best < 0)
                throw std::runtime_error("AMM needs mirror-symmetric frequency/velocity data for the interface axis "
                                         "(material " + std::to_string(m) + ", active " + std::to_string(i) + ", v " +
                                         std::to_string(x.v[0]) + "," + std::to_string(x.v[1]) + "," +
                                         std::to_string(x.v[2]) + ").");
            mirror[m][i] = best;
            mirror[m][best] = i;
        }
        for (int i = 0; i < n; ++i)
            if (std::abs(modes[m][i].v[axis]) >= 1e-7 && mirror[m][i] < 0)
                throw std::runtime_error("AMM reflection pairing is incomplete.");
    }
    // 2. each acoustic q cell, linearized, in (frequency, k_a, k_b) channel space
    std::vector<channel::M> qbasis(nm);
    std::vector<std::vector<std::unique_ptr<channel::Cell>>> cells(nm);
    for (size_t m = 0; m < nm; ++m) {
        const auto& mesh = mats[m]->q_mesh();
        const auto& rec = mats[m]->reciprocal_lattice();
        if (mesh[0] <= 0 || mesh[1] <= 0 || mesh[2] <= 0 ||
            static_cast<long long>(mesh[0]) * mesh[1] * mesh[2] != mats[m]->qpoint_count())
            throw std::runtime_error("Cell-overlap AMM requires a complete uniform q mesh.");
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) qbasis[m][i][j] = rec[i][j] / mesh[j];
        cells[m].resize(modes[m].size());
        for (size_t i = 0; i < modes[m].size(); ++i) {
            const Mode& x = modes[m][i];
            if (x.branch >= 3 || std::abs(x.v[axis]) < 1e-7) continue;
            channel::M projected{};
            for (int j = 0; j < 3; ++j) {
                for (int d = 0; d < 3; ++d) projected[0][j] += x.v[d] * qbasis[m][d][j] / (2 * pi);
                projected[1][j] = qbasis[m][ta][j];
                projected[2][j] = qbasis[m][tb][j];
            }
            cells[m][i] = std::make_unique<channel::Cell>(channel::V{x.omega / (2 * pi), x.k[ta], x.k[tb]}, projected);
        }
    }
    struct Key {
        int branch, f, x, y;
        bool operator==(const Key& k) const { return std::tie(branch, f, x, y) == std::tie(k.branch, k.f, k.x, k.y); }
    };
    struct Hash {
        size_t operator()(const Key& k) const {
            size_t h = 0;
            for (int v : {k.branch, k.f, k.x, k.y}) h ^= std::hash<int>{}(v) + 0x9e3779b9 + (h << 6) + (h >> 2);
            return h;
        }
    };
    const channel::V bin{df, dk, dk};
    auto bounds = [&](const channel::Cell& c) {
        std::array<std::array<int, 2>, 3> bs{};
        long double count = 1;
        for (int j = 0; j < 3; ++j) {
            const double lo = std::floor(c.lower[j] / bin[j]), hi = std::floor(c.upper[j] / bin[j]);
            if (!std::isfinite(lo) || !std::isfinite(hi) || lo < std::numeric_limits<int>::min() ||
                hi >= std::numeric_limits<int>::max())
                throw std::runtime_error("AMM search grid is too fine; enlarge search bins (this does not change "
                                         "channel integrals).");
            bs[j] = {static_cast<int>(lo), static_cast<int>(hi)};
            count *= hi - lo + 1;
        }
        if (count > 1000000)
            throw std::runtime_error("AMM search bins create too many candidates per cell; enlarge search bins.");
        return bs;
    };
    // 3. per interface: overlaps of incoming acoustic cells of the two sides,
    //    weighted by the scalar acoustic transmission at the quadrature points
    faces.assign(nm - 1, {});
    for (size_t face = 0; face + 1 < nm; ++face) {
        AmmFace& dst = faces[face];
        std::array<std::vector<int>, 2> incoming;
        std::array<std::vector<double>, 2> load;
        for (int side = 0; side < 2; ++side) {
            const size_t m = face + side;
            dst.rows[side].assign(modes[m].size(), AmmRow{});
            load[side].assign(modes[m].size(), 0.0);
            for (size_t i = 0; i < modes[m].size(); ++i) {
                const Mode& x = modes[m][i];
                if (side == 0 ? x.v[axis] <= 1e-7 : x.v[axis] >= -1e-7) continue;
                AmmRow& r = dst.rows[side][i];
                r.reflected = mirror[m][i];
                r.flux = x.flux;
                if (r.reflected < 0) throw std::runtime_error("Missing AMM reflection partner.");
                if (cells[m][i]) incoming[side].push_back(static_cast<int>(i));
            }
        }
        // identical banks: no interface in the acoustic subspace
        bool identical = modes[face].size() == modes[face + 1].size() &&
                         mats[face]->energy_density_normalization() == mats[face + 1]->energy_density_normalization() &&
                         densities[face] == densities[face + 1];
        for (size_t i = 0; identical && i < modes[face].size(); ++i) {
            const Mode& x = modes[face][i];
            const Mode& y = modes[face + 1][i];
            if (x.omega != y.omega || x.k != y.k || x.v != y.v) identical = false;
        }
        if (identical) {
            for (int side = 0; side < 2; ++side)
                for (int i : incoming[side]) dst.rows[side][i].transmitted.push_back({i, 1.0});
            continue;
        }
        const bool direct = incoming[0].size() * incoming[1].size() <= 4096;
        std::unordered_map<Key, std::vector<int>, Hash> index;
        if (!direct) {
            for (int j : incoming[1]) {
                const auto bs = bounds(*cells[face + 1][j]);
                for (int f = bs[0][0]; f <= bs[0][1]; ++f)
                    for (int x = bs[1][0]; x <= bs[1][1]; ++x)
                        for (int y = bs[2][0]; y <= bs[2][1]; ++y) index[{modes[face + 1][j].branch, f, x, y}].push_back(j);
            }
        }
        struct Pair {
            int left, right;
            double g;
        };
        std::vector<Pair> pairs;
        std::vector<int> seen(modes[face + 1].size(), -1);
        auto impedance = [&](size_t m, int i, const channel::V& point) {
            const Mode& mode = modes[m][i];
            const channel::V local = cells[m][i]->coordinates(point);
            Vec3 k = mode.k;
            for (int d = 0; d < 3; ++d)
                for (int j = 0; j < 3; ++j) k[d] += qbasis[m][d][j] * local[j];
            const double norm = std::sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
            return std::array<double, 2>{norm > 0 ? densities[m] * point[0] * 2 * pi / norm : 0,
                                         norm > 0 ? std::abs(k[axis]) / norm : 0};
        };
        for (int i : incoming[0]) {
            const channel::Cell& c = *cells[face][i];
            std::vector<int> candidates;
            if (direct) {
                for (int j : incoming[1])
                    if (modes[face][i].branch == modes[face + 1][j].branch) candidates.push_back(j);
            } else {
                const auto bs = bounds(c);
                for (int f = bs[0][0]; f <= bs[0][1]; ++f)
                    for (int x = bs[1][0]; x <= bs[1][1]; ++x)
                        for (int y = bs[2][0]; y <= bs[2][1]; ++y) {
                            auto it = index.find({modes[face][i].branch, f, x, y});
                            if (it == index.end()) continue;
                            for (int j : it->second)
                                if (seen[j] != i) {
                                    seen[j] = i;
                                    candidates.push_back(j);
                                }
                        }
            }
            std::sort(candidates.begin(), candidates.end()); // accumulation order independent of the search grid
            for (int j : candidates) {
                const channel::Cell& other = *cells[face + 1][j];
                const auto points = channel::quadrature(channel::intersect(c, other));
                if (points.empty()) continue;
                double overlap = 0, g = 0;
                const double density = std::min(modes[face][i].flux / c.volume, modes[face + 1][j].flux / other.volume);
                for (const auto& q : points) {
                    if (q.point[0] <= 0) continue;
                    const auto z1 = impedance(face, i, q.point), z2 = impedance(face + 1, j, q.point);
                    overlap += q.weight * density;
                    if (z1[0] > 0 && z2[0] > 0)
                        g += q.weight * density * transmission(z1[0], z2[0], std::min(1., z1[1]), std::min(1., z2[1]));
                }
                if (g > 0) {
                    pairs.push_back({i, j, g});
                    load[0][i] += overlap;
                    load[1][j] += overlap;
                }
            }
        }
        // overlapping neighbour cells: bound both marginals with one factor (reciprocity)
        for (const Pair& p : pairs) {
            const double wl = modes[face][p.left].flux, wr = modes[face + 1][p.right].flux;
            const double factor = std::max({1., load[0][p.left] / wl, load[1][p.right] / wr});
            const double g = p.g / factor;
            dst.rows[0][p.left].transmitted.push_back({mirror[face + 1][p.right], g / wl});
            dst.rows[1][p.right].transmitted.push_back({mirror[face][p.left], g / wr});
        }
        for (int side = 0; side < 2; ++side)
            for (int i : incoming[side]) {
                double sum = 0;
                for (const auto& e : dst.rows[side][i].transmitted) sum += e.second;
                if (sum > 1 + 1e-10) throw std::runtime_error("AMM row exceeds unit probability.");
            }
    }
}

} // namespace phmc
