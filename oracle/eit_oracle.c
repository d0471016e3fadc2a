/*
 * eit_oracle.c -- FP64 CPU restatement of mpFlow's EIT hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the GPU library in
 * mpflow_gb300/ is checked against.  Only tests/, __graft_entry__.smoke() and
 * the CPU-baseline leg of bench.py may load it; the product never links it.
 *
 * Every routine restates one piece of the reference (pgebhardt/mpflow) and
 * cites the file:line it follows.  Arithmetic is IEEE double throughout; the
 * reference's own template instantiations run in float or double, so the
 * oracle is the double-precision instance of the same algorithm.
 *
 * Parity status: the reference ships no tests, golden vectors or fixtures and
 * cannot be built here (Eigen, libdistmesh, json-parser absent), so the host
 * routines below are pinned only by the known-answer properties in
 * tests/test_oracle.py (reciprocity, current conservation, homogeneity, FD
 * Jacobian, analytic P1 integrals).  Parity of these host routines against
 * the reference is therefore "parity unpinned".
 *
 * Layout conventions (all as in the reference):
 *   dense matrices are column-major with the row count padded by
 *   orc_data_rows() (src/numeric/matrix.cpp:49-55);
 *   the ELL sparse format has 32 slots per row, row-major
 *   values[row*32+slot], unused slots hold column id 0xFFFFFFFF
 *   (include/mpflow/numeric/constants.h:28-33, include/mpflow/constants.h:30).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_ELL_WIDTH 32u
#define ORC_BLOCK 16u
#define ORC_INVALID 0xFFFFFFFFu

/* status codes shared with the library's mpf_status */
#define ORC_OK 0
#define ORC_EINVAL 1
#define ORC_ENOMEM 2
#define ORC_EFULL 7

/* ------------------------------------------------------------------------ */
/* padding rules                                                             */
/* ------------------------------------------------------------------------ */

/* include/mpflow/mathematics.h:42-44 (roundTo) and src/numeric/matrix.cpp:49-55:
 * a dimension is padded to the next multiple of 16 *strictly above* it unless
 * it already is a multiple of 16 or equals 1. */
unsigned orc_data_rows(unsigned rows) {
    if (rows % ORC_BLOCK != 0 && rows != 1) {
        return rows == 0 ? 0 : (rows / ORC_BLOCK + 1) * ORC_BLOCK;
    }
    return rows;
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* mesh topology: edge table and boundary                                    */
/* ------------------------------------------------------------------------ */

/* The reference delegates edges to libdistmesh (findUniqueEdges,
 * getTriangulationEdgeIndices, fixBoundaryEdgeOrientation, boundEdges;
 * src/numeric/irregular_mesh.cpp:25-46).  libdistmesh is not available, so the
 * numbering here is this project's own deterministic convention, shared with
 * the library:
 *   - elements are scanned in order, local edges in the order (0,1),(1,2),(2,0);
 *   - a new edge gets the next index and is stored (min node, max node);
 *   - an edge seen by exactly one element is a boundary edge; it is re-oriented
 *     to follow its element counter-clockwise (interior on the left), which is
 *     the orientation circularBoundary relies on (src/fem/ports.cpp:51-63);
 *   - boundary lists boundary edge indices in increasing order.
 * Returns the number of edges, or -1 on bad input. */
/* Concentric-ring disk, the workload mesh of the benchmark (no reference
 * counterpart: the reference meshes with libdistmesh, which is absent).
 * Node 0 is the centre; ring i (1..R) carries 6i nodes at radius
 * radius*i/R, angles 2 pi k / (6i), numbered 1 + 3i(i-1) + k.  Triangles: the
 * six around the centre, then for every ring i >= 2 and sector s the strip
 * between rings i-1 and i (outer edge j, then the inner edge after it),
 * each oriented counter-clockwise.  Returns the element count. */
static int orc_ring_node(int ring, int k) { return ring == 0 ? 0 : 1 + 3 * ring * (ring - 1) + k % (6 * ring); }

static void orc_ring_tri(const double* nodes, int* elements, int* e, int a, int b, int c) {
    const double ax = nodes[2 * a], ay = nodes[2 * a + 1];
    const double orient = (nodes[2 * b] - ax) * (nodes[2 * c + 1] - ay) - (nodes[2 * c] - ax) * (nodes[2 * b + 1] - ay);
    int* t = elements + 3 * (*e);
    t[0] = a;
    t[1] = orient < 0.0 ? c : b;
    t[2] = orient < 0.0 ? b : c;
    ++(*e);
}

int orc_ring_mesh(int R, double radius, double* nodes, int* elements) {
    if (R < 1 || !(radius > 0.0)) return -1;
    nodes[0] = nodes[1] = 0.0;
    for (int i = 1; i <= R; ++i) {
        const double r = radius * (double)i / (double)R;
        for (int k = 0; k < 6 * i; ++k) {
            const double th = (2.0 * M_PI * (double)k) / (6.0 * (double)i);
            const int id = orc_ring_node(i, k);
            nodes[2 * id] = r * cos(th);
            nodes[2 * id + 1] = r * sin(th);
        }
    }
    int e = 0;
    for (int k = 0; k < 6; ++k) orc_ring_tri(nodes, elements, &e, 0, orc_ring_node(1, k), orc_ring_node(1, k + 1));
    for (int i = 2; i <= R; ++i)
        for (int sct = 0; sct < 6; ++sct)
            for (int j = 0; j < i; ++j) {
                const int in0 = orc_ring_node(i - 1, sct * (i - 1) + j);
                const int o0 = orc_ring_node(i, sct * i + j), o1 = orc_ring_node(i, sct * i + j + 1);
                orc_ring_tri(nodes, elements, &e, in0, o0, o1);
                if (j < i - 1) orc_ring_tri(nodes, elements, &e, in0, o1, orc_ring_node(i - 1, sct * (i - 1) + j + 1));
            }
    return e;
}

int orc_mesh_edges(int N, int E, const double* nodes, const int* elements,
                   int* edges /* cap 3E x 2 */, int* elementEdges /* E x 3 */,
                   int* boundary /* cap 3E */, int* nBoundary) {
    if (N <= 0 || E <= 0) return -1;
    /* adjacency: for node a, list of (b, edge) with a < b */
    int* head = (int*)malloc(sizeof(int) * (size_t)N);
    int* next = (int*)malloc(sizeof(int) * (size_t)(3 * E));
    int* other = (int*)malloc(sizeof(int) * (size_t)(3 * E));
    int* count = (int*)calloc((size_t)(3 * E), sizeof(int));
    int* owner = (int*)malloc(sizeof(int) * (size_t)(3 * E));
    int* ownerLocal = (int*)malloc(sizeof(int) * (size_t)(3 * E));
    if (!head || !next || !other || !count || !owner || !ownerLocal) return -1;
    for (int i = 0; i < N; ++i) head[i] = -1;
    int nEdges = 0;
    for (int e = 0; e < E; ++e) {
        for (int l = 0; l < 3; ++l) {
            int a = elements[3 * e + l], b = elements[3 * e + (l + 1) % 3];
            if (a < 0 || a >= N || b < 0 || b >= N) return -1;
            int lo = a < b ? a : b, hi = a < b ? b : a;
            int found = -1;
            for (int it = head[lo]; it >= 0; it = next[it]) {
                if (other[it] == hi) { found = it; break; }
            }
            if (found < 0) {
                found = nEdges++;
                other[found] = hi;
                next[found] = head[lo];
                head[lo] = found;
                edges[2 * found] = lo;
                edges[2 * found + 1] = hi;
                owner[found] = e;
                ownerLocal[found] = l;
            }
            count[found] += 1;
            elementEdges[3 * e + l] = found;
        }
    }
    int nb = 0;
    for (int k = 0; k < nEdges; ++k) {
        if (count[k] == 1) {
            int e = owner[k], l = ownerLocal[k];
            const int* el = &elements[3 * e];
            double x0 = nodes[2 * el[0]], y0 = nodes[2 * el[0] + 1];
            double x1 = nodes[2 * el[1]], y1 = nodes[2 * el[1] + 1];
            double x2 = nodes[2 * el[2]], y2 = nodes[2 * el[2] + 1];
            double det = (x1 - x0) * (y2 - y0) - (x2 - x0) * (y1 - y0);
            int a = el[l], b = el[(l + 1) % 3];
            if (det < 0.0) { int t = a; a = b; b = t; }
            edges[2 * k] = a;
            edges[2 * k + 1] = b;
            boundary[nb++] = k;
        }
    }
    *nBoundary = nb;
    free(head); free(next); free(other); free(count); free(owner); free(ownerLocal);
    return nEdges;
}

/* ------------------------------------------------------------------------ */
/* circular ports                                                            */
/* ------------------------------------------------------------------------ */

/* src/mathematics.cpp:24-52 (math::polar): radius and quadrant-corrected atan. */
static void orc_polar(double x, double y, double* radius, double* angle) {
    double a;
    double r = sqrt(x * x + y * y);
    if (x > 0.0) a = atan(y / x);
    else if (x < 0.0 && y >= 0.0) a = atan(y / x) + M_PI;
    else if (x < 0.0 && y < 0.0) a = atan(y / x) - M_PI;
    else if (x == 0.0 && y > 0.0) a = M_PI / 2.0;
    else if (x == 0.0 && y < 0.0) a = -M_PI / 2.0;
    else a = 0.0;
    *radius = r;
    *angle = a;
}

/* src/mathematics.cpp:64-77 (math::circleParameter): arc parameter of a point
 * measured from an arc offset, wrapped to (-pi, pi]. */
static double orc_circle_parameter(double x, double y, double offset) {
    double r, angle;
    orc_polar(x, y, &r, &angle);
    angle -= offset / r;
    angle += (angle < -M_PI) ? 2.0 * M_PI : 0.0;
    angle -= (angle > M_PI) ? 2.0 * M_PI : 0.0;
    return angle * r;
}

/* src/mathematics.cpp:79-89 (math::arange) and :91-100 (math::circularPoints)
 * restated for a circle centred at the origin.  Returns the number of points. */
static unsigned orc_circular_points(double radius, double distance, double offset,
                                    int invert, double* xy, unsigned cap) {
    double start = offset / radius, end = offset / radius + 2.0 * M_PI;
    double step = distance / radius;
    unsigned n = (unsigned)ceil((end - start) / step);
    for (unsigned i = 0; i < n && i < cap; ++i) {
        double phi = start + (double)i * step;
        xy[2 * i] = 0.0 + radius * cos(phi);
        xy[2 * i + 1] = 0.0 + (invert ? -1.0 : 1.0) * radius * sin(phi);
    }
    return n;
}

/* src/fem/ports.cpp:32-77 (Ports::circularBoundary).  portEdges is count x cap
 * row-major, unused entries -1 (the reference pads with invalidIndex cast to
 * int, which is -1).  Returns ORC_OK or ORC_EINVAL. */
int orc_circular_ports(int N, const double* nodes, int E, const int* elements,
                       const int* edges, int nBoundary, const int* boundary,
                       int count, double width, double offset, int clockwise,
                       int* portEdges, int cap, int* maxPortEdges) {
    if (count <= 0 || N <= 0 || E <= 0) return ORC_EINVAL;
    double radius = 0.0;
    for (int e = 0; e < E; ++e) {
        for (int l = 0; l < 3; ++l) {
            int n = elements[3 * e + l];
            double x = nodes[2 * n], y = nodes[2 * n + 1];
            double r = sqrt(x * x + y * y);
            radius = radius > r ? radius : r;
        }
    }
    unsigned pcap = (unsigned)count + 4;
    double* ps = (double*)malloc(sizeof(double) * 2 * pcap);
    double* pe = (double*)malloc(sizeof(double) * 2 * pcap);
    unsigned ns = orc_circular_points(radius, 2.0 * M_PI * radius / count,
                                      offset + (clockwise ? width : 0.0), clockwise, ps, pcap);
    unsigned ne = orc_circular_points(radius, 2.0 * M_PI * radius / count,
                                      offset + (clockwise ? 0.0 : width), clockwise, pe, pcap);
    if (ns < (unsigned)count || ne < (unsigned)count) { free(ps); free(pe); return ORC_EINVAL; }
    for (int i = 0; i < count * cap; ++i) portEdges[i] = -1;
    int maxEdges = 0;
    for (int port = 0; port < count; ++port) {
        int k = 0;
        for (int b = 0; b < nBoundary; ++b) {
            int edge = boundary[b];
            int n0 = edges[2 * edge], n1 = edges[2 * edge + 1];
            double x0 = nodes[2 * n0], y0 = nodes[2 * n0 + 1];
            double x1 = nodes[2 * n1], y1 = nodes[2 * n1 + 1];
            double p0 = sqrt((x0 - x0) * (x0 - x0) + (y0 - y0) * (y0 - y0));
            double p1 = sqrt((x1 - x0) * (x1 - x0) + (y1 - y0) * (y1 - y0));
            double parameterOffset = orc_circle_parameter(x0, y0, 0.0);
            double intervalStart = orc_circle_parameter(ps[2 * port], ps[2 * port + 1], parameterOffset);
            double intervalEnd = orc_circle_parameter(pe[2 * port], pe[2 * port + 1], parameterOffset);
            if (intervalStart < intervalEnd && p0 - intervalStart >= -1e-9 &&
                p1 - intervalEnd <= 1e-9) {
                if (k >= cap) { free(ps); free(pe); return ORC_EFULL; }
                portEdges[port * cap + k] = edge;
                ++k;
                maxEdges = maxEdges > k ? maxEdges : k;
            }
        }
    }
    *maxPortEdges = maxEdges;
    free(ps);
    free(pe);
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* P1 elemental integrals                                                    */
/* ------------------------------------------------------------------------ */

/* include/mpflow/mathematics.h:55-110 (gaussElemination): 3x3 Gaussian
 * elimination with partial pivoting, used by the P1 basis constructor
 * (src/fem/basis_linear.cpp:27-56) to get phi_one = c0 + c1 x + c2 y. */
static void orc_gauss3(double A[3][3], double b[3]) {
    const int n = 3;
    for (int k = 0; k < n - 1; ++k) {
        int piv = k;
        for (int i = k; i < n; ++i) piv = fabs(A[i][k]) > fabs(A[piv][k]) ? i : piv;
        for (int i = 0; i < n; ++i) { double t = A[piv][i]; A[piv][i] = A[k][i]; A[k][i] = t; }
        { double t = b[piv]; b[piv] = b[k]; b[k] = t; }
        for (int i = k + 1; i < n; ++i) {
            double x = A[i][k] / A[k][k];
            for (int j = k; j < n; ++j) A[i][j] = A[i][j] - A[k][j] * x;
            b[i] = b[i] - b[k] * x;
        }
    }
    b[n - 1] = b[n - 1] / A[n - 1][n - 1];
    for (int i = n - 2; i >= 0; --i) {
        double s = b[i];
        for (int j = i + 1; j < n; ++j) s = s - A[i][j] * b[j];
        b[i] = s / A[i][i];
    }
}

/* Elemental stiffness K_e[i][j] = int grad(phi_i).grad(phi_j) and mass
 * M_e[i][j] = int phi_i phi_j over each triangle, row-major 3x3 per element.
 * Follows src/fem/basis_linear.cpp:72-91 (integralB / integralA): the
 * reference evaluates the symbolic integrals of the P1 polynomials times
 * |det|; the stiffness is 0.5*|det|*(c1_i c1_j + c2_i c2_j) and the symbolic
 * mass integral equals the analytic |det|/24*(1+delta_ij). */
void orc_p1_elemental(int E, const double* nodes, const int* elements, double* K, double* M) {
    #pragma omp parallel for schedule(static)
    for (int e = 0; e < E; ++e) {
        double px[3], py[3], c[3][3];
        for (int l = 0; l < 3; ++l) {
            px[l] = nodes[2 * elements[3 * e + l]];
            py[l] = nodes[2 * elements[3 * e + l] + 1];
        }
        for (int one = 0; one < 3; ++one) {
            double A[3][3], b[3] = {0.0, 0.0, 0.0};
            b[one] = 1.0;
            for (int l = 0; l < 3; ++l) { A[l][0] = 1.0; A[l][1] = px[l]; A[l][2] = py[l]; }
            orc_gauss3(A, b);
            c[one][0] = b[0]; c[one][1] = b[1]; c[one][2] = b[2];
        }
        double det = fabs((-px[0] + px[1]) * (-py[0] + py[2]) - (-px[0] + px[2]) * (-py[0] + py[1]));
        for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 3; ++j) {
                K[9 * e + 3 * i + j] = (0.5 * c[i][1] * c[j][1] + 0.5 * c[i][2] * c[j][2]) * det;
                M[9 * e + 3 * i + j] = det / 24.0 * (i == j ? 2.0 : 1.0);
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* ELL layout and level decomposition                                        */
/* ------------------------------------------------------------------------ */

/* src/numeric/sparse_matrix.cpp:358-376 (getColumnId): slot holding col, or
 * invalid. */
static unsigned orc_ell_slot(const uint32_t* ids, unsigned row, unsigned col) {
    for (unsigned i = 0; i < ORC_ELL_WIDTH; ++i)
        if (ids[row * ORC_ELL_WIDTH + i] == col) return i;
    return ORC_INVALID;
}

/* src/numeric/sparse_matrix.cpp:396-423 (setValue): the first free slot takes
 * a new column, density tracks the highest used slot; a full row is an error. */
static int orc_ell_insert(uint32_t* ids, unsigned* density, unsigned row, unsigned col, unsigned* slot) {
    for (unsigned i = 0; i < ORC_ELL_WIDTH; ++i) {
        uint32_t c = ids[row * ORC_ELL_WIDTH + i];
        if (c == col) { *slot = i; return ORC_OK; }
        if (c == ORC_INVALID) {
            ids[row * ORC_ELL_WIDTH + i] = col;
            if (i + 1 > *density) *density = i + 1;
            *slot = i;
            return ORC_OK;
        }
    }
    return ORC_EFULL;
}

/* Number of levels (maximum number of elements sharing one matrix entry):
 * the length of the connectivityMatrices vector built in
 * src/fem/equation.cpp:88-128. */
int orc_equation_levels(int N, int E, const int* elements) {
    unsigned dataRows = orc_data_rows((unsigned)N);
    uint32_t* ids = (uint32_t*)malloc(sizeof(uint32_t) * dataRows * ORC_ELL_WIDTH);
    unsigned* cnt = (unsigned*)calloc((size_t)dataRows * ORC_ELL_WIDTH, sizeof(unsigned));
    unsigned density = 0, levels = 0;
    for (size_t i = 0; i < (size_t)dataRows * ORC_ELL_WIDTH; ++i) ids[i] = ORC_INVALID;
    for (int e = 0; e < E; ++e)
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                unsigned slot, r = (unsigned)elements[3 * e + i], c = (unsigned)elements[3 * e + j];
                if (orc_ell_insert(ids, &density, r, c, &slot) != ORC_OK) { free(ids); free(cnt); return -ORC_EFULL; }
                unsigned lv = cnt[r * ORC_ELL_WIDTH + slot]++;
                if (lv + 1 > levels) levels = lv + 1;
            }
    free(ids);
    free(cnt);
    return (int)levels;
}

/* src/fem/equation.cpp:76-176 (Equation::initElementalMatrices).
 *   colIds     dataRows x 32 row-major: the commonElementMatrix layout, slot
 *              order = first insertion in the (element, i, j) loop (:131-138);
 *              copied into sMatrix, rMatrix and systemMatrix (:142-144);
 *   connectivity, elemS, elemR: dataRows x (32*levels) column-major
 *              (:147-172); entry (row, level*32+slot) is the element that is
 *              the level-th (in element order) to touch that matrix entry,
 *              with its stiffness / mass integral; absent entries are
 *              0xFFFFFFFF / 0.
 * K, M are the per-element integrals from orc_p1_elemental. */
int orc_equation_layout(int N, int E, const int* elements, const double* K, const double* M,
                        unsigned levels, uint32_t* colIds, unsigned* density,
                        uint32_t* connectivity, double* elemS, double* elemR) {
    unsigned dataRows = orc_data_rows((unsigned)N);
    size_t nslot = (size_t)dataRows * ORC_ELL_WIDTH;
    for (size_t i = 0; i < nslot; ++i) colIds[i] = ORC_INVALID;
    for (size_t i = 0; i < nslot * levels; ++i) { connectivity[i] = ORC_INVALID; elemS[i] = 0.0; elemR[i] = 0.0; }
    unsigned* cnt = (unsigned*)calloc(nslot, sizeof(unsigned));
    unsigned dens = 0;
    /* common element matrix: insertion order of the (element, i, j) loop */
    for (int e = 0; e < E; ++e)
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                unsigned slot;
                if (orc_ell_insert(colIds, &dens, (unsigned)elements[3 * e + i],
                                   (unsigned)elements[3 * e + j], &slot) != ORC_OK) {
                    free(cnt);
                    return ORC_EFULL;
                }
            }
    /* levels: the level-th element (in element order) touching (row, col) */
    for (int e = 0; e < E; ++e)
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) {
                unsigned r = (unsigned)elements[3 * e + i], c = (unsigned)elements[3 * e + j];
                unsigned slot = orc_ell_slot(colIds, r, c);
                unsigned lv = cnt[r * ORC_ELL_WIDTH + slot]++;
                if (lv >= levels) { free(cnt); return ORC_EINVAL; }
                size_t idx = (size_t)r + (size_t)(lv * ORC_ELL_WIDTH + slot) * dataRows;
                connectivity[idx] = (uint32_t)e;
                elemS[idx] = K[9 * e + 3 * i + j];
                elemR[idx] = M[9 * e + 3 * i + j];
            }
    *density = dens;
    free(cnt);
    return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* assembly                                                                  */
/* ------------------------------------------------------------------------ */

/* src/fem/equation_kernel.cu:35-53 (matParam / matParamDeriv): linear or the
 * dB-like logarithmic parametrisation sigma = ref * 10^(v/10). */
static double orc_mat_param(double ref, double v, int logarithmic) {
    return logarithmic ? ref * exp(log(10.0) * v / 10.0) : ref * v;
}
static double orc_mat_param_deriv(double ref, double v, int logarithmic) {
    return logarithmic ? (log(10.0) / 10.0) * ref * exp(log(10.0) * v / 10.0) : ref;
}

/* src/fem/equation_kernel.cu:60-82 (updateMatrixKernel): every ELL slot
 * (row, slot) sums elemental[row, slot+32*level] * matParam(gamma[element])
 * over the levels in order.  values is dataRows x 32 row-major. */
void orc_update_matrix(unsigned dataRows, unsigned levels, const uint32_t* connectivity,
                       const double* elemental, const double* gamma, double ref, int logarithmic,
                       double* values) {
    #pragma omp parallel for schedule(static)
    for (long row = 0; row < (long)dataRows; ++row) {
        for (unsigned col = 0; col < ORC_ELL_WIDTH; ++col) {
            double v = 0.0;
            for (unsigned k = 0; k < levels; ++k) {
                size_t idx = (size_t)row + (size_t)(col + k * ORC_ELL_WIDTH) * dataRows;
                uint32_t el = connectivity[idx];
                v += el != ORC_INVALID ? elemental[idx] * orc_mat_param(ref, gamma[el], logarithmic) : 0.0;
            }
            values[(size_t)row * ORC_ELL_WIDTH + col] = v;
        }
    }
}

/* src/fem/equation_kernel.cu:137-157 (updateSystemMatrixKernel):
 * sys = S + k * R on the used slots, untouched elsewhere. */
void orc_update_system_matrix(unsigned dataRows, const double* s, const double* r,
                              const uint32_t* colIds, unsigned density, double k, double* sys) {
    for (unsigned row = 0; row < dataRows; ++row)
        for (unsigned c = 0; c < density; ++c) {
            size_t idx = (size_t)row * ORC_ELL_WIDTH + c;
            if (colIds[idx] != ORC_INVALID) sys[idx] = s[idx] + r[idx] * k;
        }
}

/* ------------------------------------------------------------------------ */
/* excitation matrix                                                         */
/* ------------------------------------------------------------------------ */

/* src/fem/equation.cpp:183-215 (initExcitationMatrix) with the P1 boundary
 * integral of src/fem/basis_linear.cpp:95-124: over an edge of length L the
 * hat function of either end node integrates to L/2; every port column is
 * normalised by the port's total edge length.  exc is dataRows x count
 * column-major (leading dimension ldExc). */
void orc_excitation_matrix(int N, const double* nodes, const int* edges, int count,
                           const int* portEdges, int cap, double* exc, int ldExc) {
    for (int i = 0; i < ldExc * count; ++i) exc[i] = 0.0;
    (void)N;
    for (int port = 0; port < count; ++port) {
        double portLength = 0.0;
        int ne = 0;
        while (ne < cap && portEdges[port * cap + ne] != -1) ++ne;
        for (int k = 0; k < ne; ++k) {
            int edge = portEdges[port * cap + k];
            int a = edges[2 * edge], b = edges[2 * edge + 1];
            double dx = nodes[2 * b] - nodes[2 * a], dy = nodes[2 * b + 1] - nodes[2 * a + 1];
            portLength += sqrt(dx * dx + dy * dy);
        }
        for (int k = 0; k < ne; ++k) {
            int edge = portEdges[port * cap + k];
            int a = edges[2 * edge], b = edges[2 * edge + 1];
            double dx = nodes[2 * b] - nodes[2 * a], dy = nodes[2 * b + 1] - nodes[2 * a + 1];
            double L = sqrt(dx * dx + dy * dy);
            /* boundaryIntegral(parameter={0, L}, node): c0 = 1, c1 = -1/L,
             * integral = L*c0 + L^2*c1/2 = L/2 for both nodes */
            double c0 = (1.0 * 0.0) / ((-1.0 * 0.0) + (1.0 * L)) + 1.0;
            double c1 = -1.0 / ((-1.0 * 0.0) + (1.0 * L));
            double integral = (-(0.0 * 0.0) * c1) / 2 - 0.0 * c0 + (L * L * c1) / 2 + L * c0;
            exc[a + port * ldExc] += integral / portLength;
            exc[b + port * ldExc] += integral / portLength;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* sparse products and the preconditioned conjugate gradient                 */
/* ------------------------------------------------------------------------ */

/* src/numeric/sparse_matrix_kernel.cu:157-196 (multiplyKernel): column by
 * column y = A x over the first `density` slots.  x, y are n x cols with
 * leading dimension ld. */
void orc_ell_multiply(unsigned n, const double* values, const uint32_t* colIds, unsigned density,
                      const double* x, unsigned ld, unsigned cols, double* y) {
    #pragma omp parallel for schedule(static)
    for (long c = 0; c < (long)cols; ++c) {
        const double* xc = x + (size_t)c * ld;
        double* yc = y + (size_t)c * ld;
        for (unsigned row = 0; row < n; ++row) {
            double res = 0.0;
            for (unsigned j = 0; j < density; ++j) {
                uint32_t id = colIds[(size_t)row * ORC_ELL_WIDTH + j];
                res += id != ORC_INVALID ? xc[id] * values[(size_t)row * ORC_ELL_WIDTH + j] : 0.0;
            }
            yc[row] = res;
        }
    }
}

/* Restatement of src/numeric/conjugate_gradient.cpp:61-161 for one column
 * (the reference keeps one set of scalars per column, so columns are
 * independent), with the Jacobi preconditioner of
 * src/numeric/preconditioner_kernel.cu:63-83 (z = r / A_ii) and the dcFree
 * regularisation of :85-89 and :115-119 (the column sum of the vector is
 * added to every row).  The update guards of
 * src/numeric/conjugate_gradient_kernel.cu:77-89 (a zero denominator yields a
 * zero result) are kept.  The reference stops when sqrt(r.z / b.b) falls
 * below the machine epsilon of its type on column 0; here every column stops
 * on its own at sqrt(r.z / b.b) < tol, since parity is judged on converged
 * solutions.  Returns the iteration count. */
static unsigned orc_pcg_column(unsigned n, const double* values, const uint32_t* colIds, unsigned density,
                               const double* diagInv, const double* b, double* x, double tol,
                               unsigned maxIter, int dcFree, double* work) {
    double *r = work, *z = work + n, *p = work + 2 * n, *t = work + 3 * n;
    unsigned iterations = maxIter == 0 ? 10 * n : maxIter;
    for (unsigned row = 0; row < n; ++row) {
        double res = 0.0;
        for (unsigned j = 0; j < density; ++j) {
            uint32_t id = colIds[(size_t)row * ORC_ELL_WIDTH + j];
            res += id != ORC_INVALID ? x[id] * values[(size_t)row * ORC_ELL_WIDTH + j] : 0.0;
        }
        r[row] = -res + b[row];
    }
    if (dcFree) {
        double s = 0.0;
        for (unsigned row = 0; row < n; ++row) s += x[row];
        for (unsigned row = 0; row < n; ++row) r[row] += s;
    }
    double rzOld = 0.0, bb = 0.0;
    for (unsigned row = 0; row < n; ++row) {
        z[row] = diagInv[row] * r[row];
        p[row] = z[row];
        rzOld += r[row] * z[row];
        bb += b[row] * b[row];
    }
    if (bb == 0.0) {
        for (unsigned row = 0; row < n; ++row) x[row] = 0.0;
        return 0;
    }
    for (unsigned step = 0; step < iterations; ++step) {
        double pt = 0.0;
        for (unsigned row = 0; row < n; ++row) {
            double res = 0.0;
            for (unsigned j = 0; j < density; ++j) {
                uint32_t id = colIds[(size_t)row * ORC_ELL_WIDTH + j];
                res += id != ORC_INVALID ? p[id] * values[(size_t)row * ORC_ELL_WIDTH + j] : 0.0;
            }
            t[row] = res;
        }
        if (dcFree) {
            double s = 0.0;
            for (unsigned row = 0; row < n; ++row) s += p[row];
            for (unsigned row = 0; row < n; ++row) t[row] += s;
        }
        for (unsigned row = 0; row < n; ++row) pt += p[row] * t[row];
        double rz = 0.0;
        for (unsigned row = 0; row < n; ++row) {
            r[row] = pt != 0.0 ? r[row] - t[row] * rzOld / pt : 0.0;
            x[row] = pt != 0.0 ? x[row] + p[row] * rzOld / pt : 0.0;
            z[row] = diagInv[row] * r[row];
            rz += r[row] * z[row];
        }
        if (fabs(sqrt(rz / bb)) < tol) return step + 1;
        for (unsigned row = 0; row < n; ++row)
            p[row] = rzOld != 0.0 ? z[row] + p[row] * rz / rzOld : 0.0;
        rzOld = rz;
    }
    return iterations;
}

/* Jacobi-PCG over `cols` independent columns (OpenMP over columns).
 * b, x: n x cols, leading dimension ld.  iters receives per-column counts.
 * The diagonal is read from the ELL slots (preconditioner::diagonal on a
 * SparseMatrix, src/numeric/preconditioner.cpp:59-76). */
void orc_pcg(unsigned n, const double* values, const uint32_t* colIds, unsigned density,
             const double* b, double* x, unsigned ld, unsigned cols, double tol, unsigned maxIter,
             int dcFree, unsigned* iters) {
    double* diagInv = (double*)malloc(sizeof(double) * n);
    for (unsigned row = 0; row < n; ++row) {
        diagInv[row] = 0.0;
        for (unsigned j = 0; j < ORC_ELL_WIDTH; ++j)
            if (colIds[(size_t)row * ORC_ELL_WIDTH + j] == row) {
                diagInv[row] = 1.0 / values[(size_t)row * ORC_ELL_WIDTH + j];
                break;
            }
    }
    #pragma omp parallel
    {
        double* work = (double*)malloc(sizeof(double) * 4 * n);
        #pragma omp for schedule(dynamic, 1)
        for (long c = 0; c < (long)cols; ++c) {
            unsigned it = orc_pcg_column(n, values, colIds, density, diagInv, b + (size_t)c * ld,
                                         x + (size_t)c * ld, tol, maxIter, dcFree, work);
            if (iters) iters[c] = it;
        }
        free(work);
    }
    free(diagInv);
}

/* ------------------------------------------------------------------------ */
/* Jacobian                                                                  */
/* ------------------------------------------------------------------------ */

/* src/fem/equation_kernel.cu:197-245 (calcJacobianKernel) with
 * src/fem/equation.cpp:282-310 (calcJacobian): for row = driveId *
 * roundMeas + measId and element e,
 *   J[row, e] (+)= matParamDeriv(gamma_e) * sum_ij phiD[n_i] phiM[n_j] Ke[i + 3j]
 * where the elemental Jacobian matrix holds the stiffness integrals
 * (calculatesPotential = true, equation.cpp:240-247).  phi is n x
 * (driveCount + measCount) with leading dimension ld; J is rowsJ x E
 * column-major. */
void orc_calc_jacobian(unsigned E, const int* elements, const double* K, const double* phi,
                       unsigned ld, unsigned driveCount, unsigned measCount, const double* gamma,
                       double ref, int logarithmic, int additive, unsigned rowsJ, double* J) {
    unsigned roundMeas = ((measCount + ORC_BLOCK - 1) / ORC_BLOCK) * ORC_BLOCK;
    const double* measPhi = phi + (size_t)driveCount * ld;
    #pragma omp parallel for schedule(static)
    for (long e = 0; e < (long)E; ++e) {
        double deriv = orc_mat_param_deriv(ref, gamma[e], logarithmic);
        for (unsigned row = 0; row < rowsJ; ++row) {
            unsigned measId = row % roundMeas, driveId = row / roundMeas;
            double dPhi[3], mPhi[3];
            for (int i = 0; i < 3; ++i) {
                unsigned idx = (unsigned)elements[3 * e + i];
                dPhi[i] = driveId < driveCount ? phi[idx + (size_t)driveId * ld] : 0.0;
                mPhi[i] = measId < measCount ? measPhi[idx + (size_t)measId * ld] : 0.0;
            }
            double el = 0.0;
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                    el += dPhi[i] * mPhi[j] * K[9 * e + i + 3 * j];
            el *= deriv;
            double* dst = &J[(size_t)row + (size_t)e * rowsJ];
            *dst = additive ? *dst + el : el;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* dense kernels for the inverse problem                                     */
/* ------------------------------------------------------------------------ */

/* src/models/eit.cpp:220-245 (applyMeasurementPattern):
 * V[m, d] (+)= sum_n Att[m, n] * phi[n, d] with Att = meas^T Exc^T
 * (eit.cpp:93-94).  att is measCount x n row-major here; V is measCount x
 * driveCount column-major with leading dimension ldV. */
void orc_apply_measurement(unsigned n, unsigned measCount, unsigned driveCount, const double* att,
                           const double* phi, unsigned ld, int additive, double* V, unsigned ldV) {
    for (unsigned d = 0; d < driveCount; ++d)
        for (unsigned m = 0; m < measCount; ++m) {
            double s = 0.0;
            for (unsigned i = 0; i < n; ++i) s += att[(size_t)m * n + i] * phi[i + (size_t)d * ld];
            V[m + d * ldV] = additive ? V[m + d * ldV] + s : s;
        }
}

/* C = A^T A for A rows x cols column-major (the reference's J^T J,
 * src/solver/inverse.cpp:136-156).  C is cols x cols column-major. */
void orc_gram_t(unsigned rows, unsigned cols, const double* A, double* C) {
    #pragma omp parallel for schedule(dynamic, 8)
    for (long j = 0; j < (long)cols; ++j)
        for (unsigned i = 0; i <= (unsigned)j; ++i) {
            double s = 0.0;
            const double* ai = A + (size_t)i * rows;
            const double* aj = A + (size_t)j * rows;
            for (unsigned k = 0; k < rows; ++k) s += ai[k] * aj[k];
            C[i + (size_t)j * cols] = s;
            C[j + (size_t)i * cols] = s;
        }
}

/* C = A A^T for A rows x cols column-major (the dual-form J J^T).  C is rows
 * x rows. */
void orc_gram_n(unsigned rows, unsigned cols, const double* A, double* C) {
    for (size_t i = 0; i < (size_t)rows * rows; ++i) C[i] = 0.0;
    #pragma omp parallel
    {
        double* acc = (double*)calloc((size_t)rows * rows, sizeof(double));
        #pragma omp for schedule(static)
        for (long e = 0; e < (long)cols; ++e) {
            const double* a = A + (size_t)e * rows;
            for (unsigned j = 0; j < rows; ++j) {
                double aj = a[j];
                if (aj == 0.0) continue;
                for (unsigned i = 0; i <= j; ++i) acc[i + (size_t)j * rows] += a[i] * aj;
            }
        }
        #pragma omp critical
        for (unsigned j = 0; j < rows; ++j)
            for (unsigned i = 0; i <= j; ++i) C[i + (size_t)j * rows] += acc[i + (size_t)j * rows];
        free(acc);
    }
    for (unsigned j = 0; j < rows; ++j)
        for (unsigned i = 0; i < j; ++i) C[j + (size_t)i * rows] = C[i + (size_t)j * rows];
}

/* Dense conjugate gradient on an SPD n x n column-major matrix without a
 * preconditioner, as Inverse::solve runs it (src/solver/inverse.cpp:213-238
 * calling ConjugateGradient::solve<Matrix, Matrix> with KInv = nullptr). */
unsigned orc_dense_cg(unsigned n, const double* A, const double* b, double* x, double tol, unsigned maxIter) {
    double *r = (double*)malloc(sizeof(double) * n), *p = (double*)malloc(sizeof(double) * n),
           *t = (double*)malloc(sizeof(double) * n);
    unsigned iterations = maxIter == 0 ? 10 * n : maxIter, it = iterations;
    double bb = 0.0, rr = 0.0;
    for (unsigned i = 0; i < n; ++i) {
        double s = 0.0;
        for (unsigned k = 0; k < n; ++k) s += A[i + (size_t)k * n] * x[k];
        r[i] = b[i] - s;
        p[i] = r[i];
        bb += b[i] * b[i];
        rr += r[i] * r[i];
    }
    if (bb == 0.0) { it = 0; goto done; }
    for (unsigned step = 0; step < iterations; ++step) {
        double pt = 0.0;
        #pragma omp parallel for schedule(static) reduction(+:pt)
        for (long i = 0; i < (long)n; ++i) {
            double s = 0.0;
            for (unsigned k = 0; k < n; ++k) s += A[(size_t)i + (size_t)k * n] * p[k];
            t[i] = s;
            pt += p[i] * s;
        }
        double alpha = pt != 0.0 ? rr / pt : 0.0, rrNew = 0.0;
        for (unsigned i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            r[i] -= alpha * t[i];
            rrNew += r[i] * r[i];
        }
        if (sqrt(rrNew / bb) < tol) { it = step + 1; goto done; }
        double beta = rr != 0.0 ? rrNew / rr : 0.0;
        for (unsigned i = 0; i < n; ++i) p[i] = r[i] + beta * p[i];
        rr = rrNew;
    }
done:
    free(r); free(p); free(t);
    return it;
}

/* In-place Cholesky A = L L^T of an SPD n x n column-major matrix (lower
 * triangle overwritten by L).  Returns 0, or k+1 if the k-th pivot is not
 * positive (LAPACK's info convention). */
int orc_cholesky(unsigned n, double* A) {
    for (unsigned k = 0; k < n; ++k) {
        double d = A[k + (size_t)k * n];
        for (unsigned j = 0; j < k; ++j) d -= A[k + (size_t)j * n] * A[k + (size_t)j * n];
        if (!(d > 0.0)) return (int)k + 1;
        d = sqrt(d);
        A[k + (size_t)k * n] = d;
        #pragma omp parallel for schedule(static)
        for (long i = k + 1; i < (long)n; ++i) {
            double s = A[(size_t)i + (size_t)k * n];
            for (unsigned j = 0; j < k; ++j) s -= A[(size_t)i + (size_t)j * n] * A[k + (size_t)j * n];
            A[(size_t)i + (size_t)k * n] = s / d;
        }
    }
    return 0;
}

/* Solve L L^T x = b in place with the factor from orc_cholesky. */
void orc_cholesky_solve(unsigned n, const double* L, double* b) {
    for (unsigned i = 0; i < n; ++i) {
        double s = b[i];
        for (unsigned j = 0; j < i; ++j) s -= L[i + (size_t)j * n] * b[j];
        b[i] = s / L[i + (size_t)i * n];
    }
    for (unsigned ii = n; ii-- > 0;) {
        double s = b[ii];
        for (unsigned j = ii + 1; j < n; ++j) s -= L[j + (size_t)ii * n] * b[j];
        b[ii] = s / L[ii + (size_t)ii * n];
    }
}
