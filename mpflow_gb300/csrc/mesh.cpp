// Host-side mesh and FEM structure setup (runs once per mesh, no GPU).
//
//  * ring_mesh       -- concentric-ring disk mesh (input generator; the
//                       reference meshes with libdistmesh, which is absent)
//  * mesh_edges      -- edge table / boundary (replaces the libdistmesh utils
//                       used at src/numeric/irregular_mesh.cpp:25-46)
//  * ports_circular  -- FEM::Ports::circularBoundary, src/fem/ports.cpp:32-77
//  * p1_elemental    -- basis::Linear::integralA/B, src/fem/basis_linear.cpp:72-91
//  * build_structure -- the ELL layout of Equation::initElementalMatrices
//                       (src/fem/equation.cpp:76-176) plus this library's
//                       slot-major layout and per-slot assembly lists
//  * excitation_matrix -- Equation::initExcitationMatrix, src/fem/equation.cpp:183-215
//  * morton_order    -- this library's internal node order (no reference
//                       counterpart: the reference keeps the mesh order)
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <unordered_map>

#include "mpf_internal.h"

namespace mpf {

int ring_mesh(int R, double radius, double* nodes, int32_t* elements) {
    MPF_CHECK(R >= 1 && R <= 2000, MPF_EINVAL, "ring_mesh: rings must be in [1, 2000], got %d", R);
    MPF_CHECK(radius > 0.0, MPF_EINVAL, "ring_mesh: radius must be positive");
    auto node = [](int ring, int k) -> int32_t {
        return ring == 0 ? 0 : 1 + 3 * ring * (ring - 1) + k % (6 * ring);
    };
    nodes[0] = 0.0;
    nodes[1] = 0.0;
    for (int i = 1; i <= R; ++i) {
        double r = radius * (double)i / (double)R;
        for (int k = 0; k < 6 * i; ++k) {
            double theta = (2.0 * M_PI * (double)k) / (6.0 * (double)i);
            int32_t idx = node(i, k);
            nodes[2 * idx] = r * std::cos(theta);
            nodes[2 * idx + 1] = r * std::sin(theta);
        }
    }
    int e = 0;
    auto tri = [&](int32_t a, int32_t b, int32_t c) {
        double det = (nodes[2 * b] - nodes[2 * a]) * (nodes[2 * c + 1] - nodes[2 * a + 1]) -
                     (nodes[2 * c] - nodes[2 * a]) * (nodes[2 * b + 1] - nodes[2 * a + 1]);
        if (det < 0.0) std::swap(b, c);
        elements[3 * e] = a;
        elements[3 * e + 1] = b;
        elements[3 * e + 2] = c;
        ++e;
    };
    for (int k = 0; k < 6; ++k) tri(0, node(1, k), node(1, k + 1));
    for (int i = 2; i <= R; ++i) {
        // each of the six sectors zips i-1 inner segments with i outer ones
        for (int s = 0; s < 6; ++s) {
            for (int j = 0; j < i; ++j) {
                int32_t in0 = node(i - 1, s * (i - 1) + j);
                int32_t o0 = node(i, s * i + j), o1 = node(i, s * i + j + 1);
                tri(in0, o0, o1);
                if (j < i - 1) tri(in0, o1, node(i - 1, s * (i - 1) + j + 1));
            }
        }
    }
    return MPF_OK;
}

int mesh_edges(int N, int E, const double* nodes, const int32_t* elements, int32_t* edges,
               int32_t* elementEdges, int32_t* boundary, int32_t* nEdges, int32_t* nBoundary) {
    MPF_CHECK(N > 0 && E > 0, MPF_EINVAL, "mesh_edges: empty mesh");
    std::unordered_map<uint64_t, int32_t> index;
    index.reserve((size_t)E * 2);
    std::vector<int32_t> count, owner;
    count.reserve((size_t)E * 2);
    owner.reserve((size_t)E * 2);
    int32_t ne = 0;
    for (int e = 0; e < E; ++e) {
        for (int l = 0; l < 3; ++l) {
            int32_t a = elements[3 * e + l], b = elements[3 * e + (l + 1) % 3];
            MPF_CHECK(a >= 0 && a < N && b >= 0 && b < N && a != b, MPF_EINVAL,
                      "mesh_edges: element %d has an invalid node", e);
            int32_t lo = std::min(a, b), hi = std::max(a, b);
            uint64_t key = ((uint64_t)(uint32_t)lo << 32) | (uint32_t)hi;
            auto it = index.find(key);
            int32_t k;
            if (it == index.end()) {
                k = ne++;
                index.emplace(key, k);
                edges[2 * k] = lo;
                edges[2 * k + 1] = hi;
                count.push_back(0);
                owner.push_back(e * 3 + l);
            } else {
                k = it->second;
            }
            count[k] += 1;
            elementEdges[3 * e + l] = k;
        }
    }
    int32_t nb = 0;
    for (int32_t k = 0; k < ne; ++k) {
        if (count[k] != 1) continue;
        int e = owner[k] / 3, l = owner[k] % 3;
        const int32_t* el = elements + 3 * e;
        double ax = nodes[2 * el[0]], ay = nodes[2 * el[0] + 1];
        double det = (nodes[2 * el[1]] - ax) * (nodes[2 * el[2] + 1] - ay) -
                     (nodes[2 * el[2]] - ax) * (nodes[2 * el[1] + 1] - ay);
        int32_t a = el[l], b = el[(l + 1) % 3];
        if (det < 0.0) std::swap(a, b);
        edges[2 * k] = a;
        edges[2 * k + 1] = b;
        boundary[nb++] = k;
    }
    *nEdges = ne;
    *nBoundary = nb;
    return MPF_OK;
}

// math::polar and math::circleParameter, src/mathematics.cpp:24-77.
static void polar(double x, double y, double& r, double& angle) {
    r = std::sqrt(x * x + y * y);
    if (x > 0.0) angle = std::atan(y / x);
    else if (x < 0.0 && y >= 0.0) angle = std::atan(y / x) + M_PI;
    else if (x < 0.0 && y < 0.0) angle = std::atan(y / x) - M_PI;
    else if (x == 0.0 && y > 0.0) angle = M_PI / 2.0;
    else if (x == 0.0 && y < 0.0) angle = -M_PI / 2.0;
    else angle = 0.0;
}

static double circle_parameter(double x, double y, double offset) {
    double r, angle;
    polar(x, y, r, angle);
    angle -= offset / r;
    angle += (angle < -M_PI) ? 2.0 * M_PI : 0.0;
    angle -= (angle > M_PI) ? 2.0 * M_PI : 0.0;
    return angle * r;
}

// math::arange + math::circularPoints (src/mathematics.cpp:79-100), centred at 0.
static std::vector<double> circular_points(double radius, double distance, double offset, bool invert) {
    double start = offset / radius, end = offset / radius + 2.0 * M_PI, step = distance / radius;
    unsigned n = (unsigned)std::ceil((end - start) / step);
    std::vector<double> xy(2 * (size_t)n);
    for (unsigned i = 0; i < n; ++i) {
        double phi = start + (double)i * step;
        xy[2 * i] = 0.0 + radius * std::cos(phi);
        xy[2 * i + 1] = 0.0 + (invert ? -1.0 : 1.0) * radius * std::sin(phi);
    }
    return xy;
}

int ports_circular(int N, const double* nodes, int E, const int32_t* elements,
                   const int32_t* edges, int nBoundary, const int32_t* boundary, int count,
                   double width, double offset, int clockwise, int32_t* portEdges, int cap,
                   int32_t* maxPortEdges) {
    MPF_CHECK(count > 0 && N > 0 && E > 0 && cap > 0, MPF_EINVAL, "ports_circular: bad sizes");
    double radius = 0.0;
    for (int e = 0; e < 3 * E; ++e) {
        int32_t n = elements[e];
        MPF_CHECK(n >= 0 && n < N, MPF_EINVAL, "ports_circular: invalid element node");
        radius = std::max(radius, std::sqrt(nodes[2 * n] * nodes[2 * n] + nodes[2 * n + 1] * nodes[2 * n + 1]));
    }
    auto ps = circular_points(radius, 2.0 * M_PI * radius / count, offset + (clockwise ? width : 0.0), clockwise);
    auto pe = circular_points(radius, 2.0 * M_PI * radius / count, offset + (clockwise ? 0.0 : width), clockwise);
    MPF_CHECK(ps.size() >= 2 * (size_t)count && pe.size() >= 2 * (size_t)count, MPF_EINVAL,
              "ports_circular: degenerate port spacing");
    for (int i = 0; i < count * cap; ++i) portEdges[i] = -1;
    int32_t widest = 0;
    for (int port = 0; port < count; ++port) {
        int k = 0;
        for (int b = 0; b < nBoundary; ++b) {
            int32_t edge = boundary[b];
            int32_t n0 = edges[2 * edge], n1 = edges[2 * edge + 1];
            double x0 = nodes[2 * n0], y0 = nodes[2 * n0 + 1], x1 = nodes[2 * n1], y1 = nodes[2 * n1 + 1];
            double p0 = std::sqrt((x0 - x0) * (x0 - x0) + (y0 - y0) * (y0 - y0));
            double p1 = std::sqrt((x1 - x0) * (x1 - x0) + (y1 - y0) * (y1 - y0));
            double off = circle_parameter(x0, y0, 0.0);
            double s = circle_parameter(ps[2 * port], ps[2 * port + 1], off);
            double t = circle_parameter(pe[2 * port], pe[2 * port + 1], off);
            if (s < t && p0 - s >= -1e-9 && p1 - t <= 1e-9) {
                MPF_CHECK(k < cap, MPF_EFULL, "ports_circular: port %d has more than %d edges", port, cap);
                portEdges[port * cap + k++] = edge;
                widest = std::max(widest, (int32_t)k);
            }
        }
    }
    *maxPortEdges = widest;
    return MPF_OK;
}

void p1_elemental(int E, const double* nodes, const int32_t* elements, double* K, double* M) {
    for (int e = 0; e < E; ++e) {
        const int32_t* el = elements + 3 * e;
        double x[3], y[3];
        for (int l = 0; l < 3; ++l) {
            x[l] = nodes[2 * el[l]];
            y[l] = nodes[2 * el[l] + 1];
        }
        double det = (x[1] - x[0]) * (y[2] - y[0]) - (x[2] - x[0]) * (y[1] - y[0]);
        // gradient of the hat function of vertex l: rotated opposite edge / det
        double gx[3], gy[3];
        for (int l = 0; l < 3; ++l) {
            int a = (l + 1) % 3, b = (l + 2) % 3;
            gx[l] = (y[a] - y[b]) / det;
            gy[l] = (x[b] - x[a]) / det;
        }
        double area2 = std::fabs(det);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                K[9 * e + 3 * i + j] = 0.5 * area2 * (gx[i] * gx[j] + gy[i] * gy[j]);
                M[9 * e + 3 * i + j] = area2 / 24.0 * (i == j ? 2.0 : 1.0);
            }
    }
}

int build_structure(int N, int E, const int32_t* elements, FemStructure& fs) {
    MPF_CHECK(N > 0 && E > 0, MPF_EINVAL, "build_structure: empty mesh");
    fs.n = N;
    fs.E = E;
    fs.dataRows = (int)data_rows((uint32_t)N);
    fs.npad = round_up(N, kRowTile);
    fs.refColIds.assign((size_t)fs.dataRows * kEllWidth, kInvalid);
    // row -> ordered columns (first insertion in the element/i/j loop)
    std::vector<uint8_t> used((size_t)N, 0);
    uint32_t* ids = fs.refColIds.data();
    auto slot_of = [&](int32_t row, int32_t col, bool insert, int& slot) -> int {
        uint8_t u = used[row];
        for (int s = 0; s < u; ++s)
            if (ids[(size_t)row * kEllWidth + s] == (uint32_t)col) {
                slot = s;
                return MPF_OK;
            }
        if (!insert) return MPF_EINVAL;
        MPF_CHECK(u < kEllWidth, MPF_EFULL, "sparse format full: node %d has more than 32 neighbours", row);
        ids[(size_t)row * kEllWidth + u] = (uint32_t)col;
        used[row] = u + 1;
        slot = u;
        return MPF_OK;
    };
    for (int e = 0; e < E; ++e)
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                int32_t r = elements[3 * e + i], c = elements[3 * e + j];
                MPF_CHECK(r >= 0 && r < N && c >= 0 && c < N, MPF_EINVAL,
                          "build_structure: element %d has an invalid node", e);
                int slot;
                MPF_TRY(slot_of(r, c, true, slot));
            }
    int density = 0;
    for (int r = 0; r < N; ++r) density = std::max(density, (int)used[r]);
    fs.density = density;
    // slot-major layout with padding slots pointing at the row itself
    const int W = density, P = fs.npad;
    fs.cols.assign((size_t)W * P, 0);
    fs.diagSlot.assign((size_t)P, 0);
    for (int r = 0; r < P; ++r)
        for (int s = 0; s < W; ++s) {
            uint32_t c = (r < N && s < used[r]) ? ids[(size_t)r * kEllWidth + s] : kInvalid;
            fs.cols[(size_t)s * P + r] = c == kInvalid ? r : (int32_t)c;
            if (c == (uint32_t)r) fs.diagSlot[r] = s;
        }
    // per-slot contribution lists in element order (the reference's level order)
    std::vector<int32_t> cnt((size_t)W * P, 0);
    int levels = 0;
    for (int e = 0; e < E; ++e)
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                int32_t r = elements[3 * e + i], c = elements[3 * e + j];
                int slot = 0;
                MPF_TRY(slot_of(r, c, false, slot));  // inserted by the pass above
                int v = ++cnt[(size_t)slot * P + r];
                levels = std::max(levels, v);
            }
    fs.levels = levels;
    fs.contribPtr.assign((size_t)W * P + 1, 0);
    for (size_t s = 0; s < (size_t)W * P; ++s) fs.contribPtr[s + 1] = fs.contribPtr[s] + cnt[s];
    fs.contrib.assign((size_t)fs.contribPtr.back(), 0);
    std::vector<int32_t> fill(fs.contribPtr.begin(), fs.contribPtr.end() - 1);
    for (int e = 0; e < E; ++e)
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                int32_t r = elements[3 * e + i], c = elements[3 * e + j];
                int slot = 0;
                MPF_TRY(slot_of(r, c, false, slot));
                fs.contrib[fill[(size_t)slot * P + r]++] = e * 9 + i * 3 + j;
            }
    return MPF_OK;
}

void excitation_matrix(int N, const double* nodes, const int32_t* edges, int ports,
                       const int32_t* portEdges, int cap, double* exc, int ld) {
    (void)N;
    for (size_t i = 0; i < (size_t)ld * ports; ++i) exc[i] = 0.0;
    for (int port = 0; port < ports; ++port) {
        const int32_t* pe = portEdges + (size_t)port * cap;
        int ne = 0;
        while (ne < cap && pe[ne] != -1) ++ne;
        double portLength = 0.0;
        for (int k = 0; k < ne; ++k) {
            int32_t a = edges[2 * pe[k]], b = edges[2 * pe[k] + 1];
            double dx = nodes[2 * b] - nodes[2 * a], dy = nodes[2 * b + 1] - nodes[2 * a + 1];
            portLength += std::sqrt(dx * dx + dy * dy);
        }
        for (int k = 0; k < ne; ++k) {
            int32_t a = edges[2 * pe[k]], b = edges[2 * pe[k] + 1];
            double dx = nodes[2 * b] - nodes[2 * a], dy = nodes[2 * b + 1] - nodes[2 * a + 1];
            // the P1 hat of either end node integrates to half the edge length
            double half = 0.5 * std::sqrt(dx * dx + dy * dy);
            exc[a + (size_t)port * ld] += half / portLength;
            exc[b + (size_t)port * ld] += half / portLength;
        }
    }
}

static uint32_t spread_bits16(uint32_t v) {
    v &= 0xFFFFu;
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

void morton_order(int N, const double* nodes, int32_t* perm) {
    double x0 = 1e300, y0 = 1e300, x1 = -1e300, y1 = -1e300;
    for (int i = 0; i < N; ++i) {
        x0 = std::min(x0, nodes[2 * i]);
        x1 = std::max(x1, nodes[2 * i]);
        y0 = std::min(y0, nodes[2 * i + 1]);
        y1 = std::max(y1, nodes[2 * i + 1]);
    }
    const double span = std::max(std::max(x1 - x0, y1 - y0), 1e-300);
    std::vector<uint32_t> code(N);
    for (int i = 0; i < N; ++i) {
        const uint32_t qx = (uint32_t)std::lround((nodes[2 * i] - x0) / span * 65535.0);
        const uint32_t qy = (uint32_t)std::lround((nodes[2 * i + 1] - y0) / span * 65535.0);
        code[i] = spread_bits16(qx) | (spread_bits16(qy) << 1);
    }
    std::iota(perm, perm + N, 0);
    std::stable_sort(perm, perm + N, [&](int32_t a, int32_t b) { return code[a] < code[b]; });
}

}  // namespace mpf
