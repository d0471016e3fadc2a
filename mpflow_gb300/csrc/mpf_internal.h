// Internal declarations shared by the host setup code, the CUDA kernels and
// the C ABI layer of libmpflow_gb300.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/mpflow_gb300.h"

namespace mpf {

constexpr uint32_t kEllWidth = 32;        // reference ELL slots per row
constexpr uint32_t kBlock = 16;           // reference dense padding block
constexpr uint32_t kInvalid = 0xFFFFFFFFu;
constexpr int kRowTile = 128;             // internal node padding (CTA row tile)
constexpr int kElemTile = 64;             // internal element padding (GEMM K block)

// ---- kernel launch accounting (read by mpf_kernel_launches) -------------
void add_launches(long long n);
long long launches();

// ---- error reporting ----------------------------------------------------
void set_error(const char* fmt, ...);
int fail(int status, const char* fmt, ...);
const char* last_error();

#define MPF_CUDA(call)                                                                    \
    do {                                                                                  \
        cudaError_t mpf_e_ = (call);                                                      \
        if (mpf_e_ != cudaSuccess)                                                        \
            return ::mpf::fail(MPF_ECUDA, "%s: %s (%s:%d)", #call,                       \
                               cudaGetErrorString(mpf_e_), __FILE__, __LINE__);          \
    } while (0)

// after a kernel launch: count it and surface launch errors
#define MPF_LAUNCHED(n)                         \
    do {                                        \
        ::mpf::add_launches(n);                 \
        MPF_CUDA(cudaGetLastError());           \
    } while (0)

#define MPF_CHECK(cond, status, ...)                       \
    do {                                                   \
        if (!(cond)) return ::mpf::fail(status, __VA_ARGS__); \
    } while (0)

#define MPF_TRY(expr)                \
    do {                             \
        int mpf_s_ = (expr);         \
        if (mpf_s_ != MPF_OK) return mpf_s_; \
    } while (0)

inline uint32_t data_rows(uint32_t rows) {
    if (rows % kBlock != 0 && rows != 1) return rows == 0 ? 0 : (rows / kBlock + 1) * kBlock;
    return rows;
}
inline int round_up(int v, int m) { return (v + m - 1) / m * m; }

// ---- device buffer ------------------------------------------------------
template <class T>
struct DevBuf {
    T* ptr = nullptr;
    size_t count = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        count = 0;
    }
    int alloc(size_t n) {
        if (n <= count && ptr) return MPF_OK;
        release();
        if (n == 0) return MPF_OK;
        cudaError_t e = cudaMalloc(&ptr, n * sizeof(T));
        if (e != cudaSuccess) {
            ptr = nullptr;
            return fail(MPF_ENOMEM, "cudaMalloc(%zu bytes): %s", n * sizeof(T), cudaGetErrorString(e));
        }
        count = n;
        return MPF_OK;
    }
    int upload(const T* host, size_t n) {
        MPF_TRY(alloc(n));
        MPF_CUDA(cudaMemcpy(ptr, host, n * sizeof(T), cudaMemcpyHostToDevice));
        return MPF_OK;
    }
    int upload(const std::vector<T>& v) { return upload(v.data(), v.size()); }
};

// ---- host setup (mesh.cpp) -----------------------------------------------
int ring_mesh(int rings, double radius, double* nodes, int32_t* elements);
int mesh_edges(int N, int E, const double* nodes, const int32_t* elements, int32_t* edges,
               int32_t* elementEdges, int32_t* boundary, int32_t* nEdges, int32_t* nBoundary);
int ports_circular(int N, const double* nodes, int E, const int32_t* elements,
                   const int32_t* edges, int nBoundary, const int32_t* boundary, int count,
                   double width, double offset, int clockwise, int32_t* portEdges, int cap,
                   int32_t* maxPortEdges);
void p1_elemental(int E, const double* nodes, const int32_t* elements, double* K, double* M);

// Matrix structure of the P1 system in both layouts.
struct FemStructure {
    int n = 0, E = 0, dataRows = 0, npad = 0, density = 0, levels = 0;
    std::vector<uint32_t> refColIds;        // dataRows x 32, reference layout
    std::vector<int32_t> cols;              // density x npad slot-major (pad: col = row)
    std::vector<int32_t> diagSlot;          // npad
    std::vector<int32_t> contribPtr;        // density*npad + 1 (slot-major slot order)
    std::vector<int32_t> contrib;           // e*9 + i*3 + j, element order within a slot
};
int build_structure(int N, int E, const int32_t* elements, FemStructure& fs);
// perm[i] = node placed at row i: nodes sorted by the Morton (Z-order) code of
// their coordinates quantised to 16 bits per axis, ties by node number.
void morton_order(int N, const double* nodes, int32_t* perm);
void excitation_matrix(int N, const double* nodes, const int32_t* edges, int ports,
                       const int32_t* portEdges, int cap, double* exc, int ld);

}  // namespace mpf
