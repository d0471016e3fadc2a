// mpflow_gb300.hpp -- C++ facade with mpFlow's class names and signatures.
//
// Header-only, on top of the C ABI in mpflow_gb300.h.  It keeps the names,
// constructor and method signatures of the reference's public classes so that
// code written against them compiles with few changes:
//   numeric::Matrix<T>          include/mpflow/numeric/matrix.h
//   numeric::IrregularMesh      include/mpflow/numeric/irregular_mesh.h
//   numeric::SparseMatrix<T>    include/mpflow/numeric/sparse_matrix.h
//   numeric::ConjugateGradient  include/mpflow/numeric/conjugate_gradient.h
//   numeric::BiCGSTAB           include/mpflow/numeric/bicgstab.h
//   FEM::Ports, FEM::Sources<T> include/mpflow/fem/ports.h, sources.h
//   FEM::Equation, basis::Linear include/mpflow/fem/equation.h (template tags)
//   models::EIT<...>            include/mpflow/models/eit.h
//   solver::Inverse<...>        include/mpflow/solver/inverse.h
//   solver::Solver<...>         include/mpflow/solver/solver.h
// Differences a caller sees: Eigen arrays become numeric::Array2<T> (row-major
// host arrays with (i, j) access); cublasHandle_t parameters are accepted and
// ignored (no cuBLAS is used); failures throw the exception type the
// reference throws (std::invalid_argument for bad arguments,
// std::runtime_error otherwise) with the library's message.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <complex>
#include <cstdint>
#include <fstream>
#include <functional>
#include <iomanip>
#include <limits>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "mpflow_gb300.h"

typedef struct cublasContext* cublasHandle_t;  // accepted for signature compatibility, never used
#ifndef CUBLAS_API_H_
// the transposition flags of Matrix::multiply (values as cublas_api.h)
typedef enum { CUBLAS_OP_N = 0, CUBLAS_OP_T = 1, CUBLAS_OP_C = 2 } cublasOperation_t;
#endif

namespace mpFlow {

namespace detail {
inline void check(int status, const char* where) {
    if (status == MPF_OK) return;
    const std::string msg = std::string(where) + ": " + mpf_last_error();
    if (status == MPF_EINVAL) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}
inline void cuda(cudaError_t e, const char* where) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(where) + ": " + cudaGetErrorString(e));
}
// complex data types (thrust::complex<float>, std::complex<float>: anything
// with real() and imag(), stored as an interleaved float pair)
template <class T, class = void>
struct is_complex : std::false_type {};
template <class T>
struct is_complex<T, std::void_t<decltype(std::declval<T const&>().imag())>> : std::true_type {};
template <class T>
double real_part(T const& v) {
    if constexpr (is_complex<T>::value) return (double)v.real();
    else return (double)v;
}
template <class T>
double imag_part(T const& v) {
    if constexpr (is_complex<T>::value) return (double)v.imag();
    else return 0.0;
}
// The library computes in FP32: a real data type maps to float, a complex
// one to an interleaved float pair.  Data types of that size (float,
// thrust::complex<float>, std::complex<float>) are passed through; wider
// ones (double, complex<double>) are converted on the way in and out.
template <class T>
using lib_type = typename std::conditional<is_complex<T>::value, std::complex<float>, float>::type;
template <class T>
constexpr bool lib_native() { return sizeof(T) == sizeof(lib_type<T>); }
template <class To, class From>
To convert_value(From const& v) {
    if constexpr (is_complex<From>::value) return To(v.real(), v.imag());
    else return To(v);
}
// n values of type From on the device -> n values of type To on the device
// (one of them FP32, the other FP64, real or complex alike), stream-ordered
// on the device by mpf_convert_values
template <class To, class From>
void convert_device(To* dst, From const* src, size_t n, cudaStream_t s, const char* where) {
    static_assert(is_complex<To>::value == is_complex<From>::value, "convert_device: real <-> complex");
    if constexpr (sizeof(To) == sizeof(From)) {
        cuda(cudaMemcpyAsync(dst, src, sizeof(To) * n, cudaMemcpyDeviceToDevice, s), where);
    } else {
        const int64_t scalars = (int64_t)n * (is_complex<To>::value ? 2 : 1);
        check(mpf_convert_values(sizeof(From) > sizeof(To) ? 0 : 1, scalars, src, dst, (mpf_stream_t)s), where);
    }
}
}  // namespace detail

// Minimal JSON reader for the configuration files that the reference reads
// with json-parser (the *fromConfig factories): objects, arrays, strings,
// numbers, booleans, null.  A missing key reads as a null value, as in
// json-parser.
namespace json {
class value {
public:
    enum Type { none, object, array, string, number, boolean };
    Type type = none;
    double num = 0.0;
    bool flag = false;
    std::string str;
    std::vector<value> items;
    std::vector<std::pair<std::string, value>> members;

    const value& operator[](const std::string& key) const {
        for (auto const& kv : members)
            if (kv.first == key) return kv.second;
        return null_value();
    }
    const value& operator[](const char* key) const { return (*this)[std::string(key)]; }
    const value& operator[](size_t i) const { return i < items.size() ? items[i] : null_value(); }
    const value& operator[](int i) const { return i >= 0 ? (*this)[(size_t)i] : null_value(); }
    const value& operator[](unsigned i) const { return (*this)[(size_t)i]; }
    size_t size() const { return type == array ? items.size() : members.size(); }
    double asDouble(double def = 0.0) const { return type == number ? num : def; }
    long asInt(long def = 0) const { return type == number ? (long)std::llround(num) : def; }
    bool asBool(bool def = false) const { return type == boolean ? flag : def; }
    std::string asString(std::string const& def = "") const { return type == string ? str : def; }

    static const value& null_value() {
        static const value v;
        return v;
    }
};

inline value parse(std::string const& text) {
    size_t i = 0;
    auto fail = [&](const char* what) -> void {
        throw std::invalid_argument(std::string("mpFlow::json::parse: ") + what + " at offset " + std::to_string(i));
    };
    auto ws = [&]() {
        while (i < text.size() && (text[i] == ' ' || text[i] == '\n' || text[i] == '\t' || text[i] == '\r')) ++i;
    };
    std::function<value()> parse_value;
    auto parse_string = [&]() -> std::string {
        if (text[i] != '"') fail("string expected");
        ++i;
        std::string out;
        while (i < text.size() && text[i] != '"') {
            char c = text[i++];
            if (c == '\\' && i < text.size()) {
                const char e = text[i++];
                c = e == 'n' ? '\n' : e == 't' ? '\t' : e == 'r' ? '\r' : e == 'b' ? '\b' : e == 'f' ? '\f' : e;
            }
            out.push_back(c);
        }
        if (i >= text.size()) fail("unterminated string");
        ++i;
        return out;
    };
    parse_value = [&]() -> value {
        ws();
        if (i >= text.size()) fail("unexpected end");
        value v;
        const char c = text[i];
        if (c == '{') {
            v.type = value::object;
            ++i;
            ws();
            if (text[i] == '}') {
                ++i;
                return v;
            }
            for (;;) {
                ws();
                std::string key = parse_string();
                ws();
                if (text[i] != ':') fail("':' expected");
                ++i;
                v.members.emplace_back(key, parse_value());
                ws();
                if (text[i] == ',') {
                    ++i;
                    continue;
                }
                if (text[i] == '}') {
                    ++i;
                    return v;
                }
                fail("',' or '}' expected");
            }
        }
        if (c == '[') {
            v.type = value::array;
            ++i;
            ws();
            if (text[i] == ']') {
                ++i;
                return v;
            }
            for (;;) {
                v.items.push_back(parse_value());
                ws();
                if (text[i] == ',') {
                    ++i;
                    continue;
                }
                if (text[i] == ']') {
                    ++i;
                    return v;
                }
                fail("',' or ']' expected");
            }
        }
        if (c == '"') {
            v.type = value::string;
            v.str = parse_string();
            return v;
        }
        if (text.compare(i, 4, "true") == 0) {
            v.type = value::boolean;
            v.flag = true;
            i += 4;
            return v;
        }
        if (text.compare(i, 5, "false") == 0) {
            v.type = value::boolean;
            i += 5;
            return v;
        }
        if (text.compare(i, 4, "null") == 0) {
            i += 4;
            return v;
        }
        size_t used = 0;
        v.type = value::number;
        v.num = std::stod(text.substr(i, 64), &used);
        if (used == 0) fail("value expected");
        i += used;
        return v;
    };
    value root = parse_value();
    ws();
    if (i != text.size()) fail("trailing characters");
    return root;
}

inline value parse_file(std::string const& filename) {
    std::ifstream f(filename);
    if (!f) throw std::runtime_error("mpFlow::json::parse_file: cannot open " + filename);
    std::stringstream ss;
    ss << f.rdbuf();
    return parse(ss.str());
}
}  // namespace json

namespace math {
// include/mpflow/mathematics.h:42-44
inline unsigned roundTo(unsigned value, unsigned step) { return value == 0 ? 0 : ((value + step - 1) / step) * step; }
}  // namespace math

namespace numeric {

// Row-major host array standing in for the reference's Eigen arrays.
template <class T>
struct Array2 {
    unsigned rowsCount = 0, colsCount = 0;
    std::vector<T> data;
    Array2() = default;
    Array2(unsigned r, unsigned c, T v = T(0)) : rowsCount(r), colsCount(c), data((size_t)r * c, v) {}
    unsigned rows() const { return rowsCount; }
    unsigned cols() const { return colsCount; }
    T& operator()(unsigned i, unsigned j) { return data[(size_t)i * colsCount + j]; }
    const T& operator()(unsigned i, unsigned j) const { return data[(size_t)i * colsCount + j]; }
};

// Dense column-major matrix with padded leading dimension dataRows =
// roundTo(rows, 16) unless rows % 16 == 0 or rows == 1 (src/numeric/matrix.cpp:
// 35-97); owns a device buffer and a host copy.
template <class type>
class Matrix {
public:
    Matrix(unsigned const rows, unsigned const cols, cudaStream_t const stream = nullptr, type const value = type(0),
           bool const allocHost = true)
        : rows(rows), cols(cols), dataRows(mpf_data_rows(rows)), dataCols(mpf_data_rows(cols)) {
        if (rows == 0) throw std::invalid_argument("mpFlow::numeric::Matrix::Matrix: rows == 0");
        if (cols == 0) throw std::invalid_argument("mpFlow::numeric::Matrix::Matrix: cols == 0");
        detail::cuda(cudaMalloc((void**)&deviceData, sizeof(type) * (size_t)dataRows * dataCols),
                     "mpFlow::numeric::Matrix::Matrix: cudaMalloc");
        if (allocHost) host_.assign((size_t)dataRows * dataCols, type(0));
        fill(value, stream);
    }
    Matrix(Matrix const&) = delete;
    Matrix& operator=(Matrix const&) = delete;
    virtual ~Matrix() { cudaFree(deviceData); }

    static std::shared_ptr<Matrix<type>> eye(unsigned const size, cudaStream_t const stream = nullptr) {
        auto m = std::make_shared<Matrix<type>>(size, size, stream);
        for (unsigned i = 0; i < size; ++i) (*m)(i, i) = type(1);
        m->copyToDevice(stream);
        return m;
    }

    void copyToDevice(cudaStream_t const stream = nullptr) {
        requireHost("copyToDevice");
        detail::cuda(cudaMemcpyAsync(deviceData, host_.data(), sizeof(type) * host_.size(), cudaMemcpyHostToDevice,
                                     stream),
                     "mpFlow::numeric::Matrix::copyToDevice");
        detail::cuda(cudaStreamSynchronize(stream), "mpFlow::numeric::Matrix::copyToDevice");
    }
    void copyToHost(cudaStream_t const stream = nullptr) const {
        requireHost("copyToHost");
        detail::cuda(cudaMemcpyAsync(host_.data(), deviceData, sizeof(type) * host_.size(), cudaMemcpyDeviceToHost,
                                     stream),
                     "mpFlow::numeric::Matrix::copyToHost");
        detail::cuda(cudaStreamSynchronize(stream), "mpFlow::numeric::Matrix::copyToHost");
    }
    void fill(type const value, cudaStream_t const stream = nullptr) {
        std::vector<type> v((size_t)dataRows * dataCols, type(0));
        for (unsigned j = 0; j < cols; ++j)
            for (unsigned i = 0; i < rows; ++i) v[i + (size_t)j * dataRows] = value;
        if (!host_.empty()) host_ = v;
        detail::cuda(cudaMemcpyAsync(deviceData, v.data(), sizeof(type) * v.size(), cudaMemcpyHostToDevice, stream),
                     "mpFlow::numeric::Matrix::fill");
        detail::cuda(cudaStreamSynchronize(stream), "mpFlow::numeric::Matrix::fill");
    }
    // device-side copy of another matrix of the same shape
    void copy(std::shared_ptr<Matrix<type> const> const other, cudaStream_t const stream = nullptr) {
        if (!other || other->dataRows != dataRows || other->dataCols != dataCols)
            throw std::invalid_argument("mpFlow::numeric::Matrix::copy: shape mismatch");
        detail::cuda(cudaMemcpyAsync(deviceData, other->deviceData, sizeof(type) * (size_t)dataRows * dataCols,
                                     cudaMemcpyDeviceToDevice, stream),
                     "mpFlow::numeric::Matrix::copy");
    }

    // device arithmetic (src/numeric/matrix.cpp, FP32 matrices): through
    // mpf_matrix_elementwise / mpf_matrix_column_reduce / mpf_matrix_multiply
    void setEye(cudaStream_t const stream = nullptr) {
        if (rows != cols) throw std::invalid_argument("mpFlow::numeric::Matrix::setEye: matrix not square");
        elementwise(0, nullptr, nullptr, type(0), stream, "setEye");
    }
    void diag(std::shared_ptr<Matrix<type> const> const matrix, cudaStream_t const stream = nullptr) {
        sameShape(matrix, "diag");
        elementwise(1, matrix->deviceData, nullptr, type(0), stream, "diag");
    }
    void add(type const value, cudaStream_t const stream = nullptr) {
        elementwise(2, deviceData, nullptr, value, stream, "add");
    }
    void add(std::shared_ptr<Matrix<type> const> const value, cudaStream_t const stream = nullptr) {
        sameShape(value, "add");
        elementwise(3, deviceData, value->deviceData, type(0), stream, "add");
    }
    void scalarMultiply(type const scalar, cudaStream_t const stream = nullptr) {
        elementwise(4, deviceData, nullptr, scalar, stream, "scalarMultiply");
    }
    void elementwiseMultiply(std::shared_ptr<Matrix<type> const> const A, std::shared_ptr<Matrix<type> const> const B,
                             cudaStream_t const stream = nullptr) {
        sameShape(A, "elementwiseMultiply");
        sameShape(B, "elementwiseMultiply");
        elementwise(5, A->deviceData, B->deviceData, type(0), stream, "elementwiseMultiply");
    }
    void elementwiseDivision(std::shared_ptr<Matrix<type> const> const A, std::shared_ptr<Matrix<type> const> const B,
                             cudaStream_t const stream = nullptr) {
        sameShape(A, "elementwiseDivision");
        sameShape(B, "elementwiseDivision");
        elementwise(6, A->deviceData, B->deviceData, type(0), stream, "elementwiseDivision");
    }
    // column reductions into row 0 (src/numeric/matrix.cpp:455-660)
    void vectorDotProduct(std::shared_ptr<Matrix<type> const> const A, std::shared_ptr<Matrix<type> const> const B,
                          cudaStream_t const stream = nullptr) {
        sameShape(A, "vectorDotProduct");
        sameShape(B, "vectorDotProduct");
        reduce(1, A, B->deviceData, stream, "vectorDotProduct");
    }
    void sum(std::shared_ptr<Matrix<type> const> const value, cudaStream_t const stream = nullptr) {
        sameShape(value, "sum");
        reduce(0, value, nullptr, stream, "sum");
    }
    void min(std::shared_ptr<Matrix<type> const> const value, cudaStream_t const stream = nullptr) {
        sameShape(value, "min");
        reduce(2, value, nullptr, stream, "min");
    }
    void max(std::shared_ptr<Matrix<type> const> const value, cudaStream_t const stream = nullptr) {
        sameShape(value, "max");
        reduce(3, value, nullptr, stream, "max");
    }
    // this = op(A) op(B) (src/numeric/matrix.cpp:298-332)
    void multiply(std::shared_ptr<Matrix<type> const> const A, std::shared_ptr<Matrix<type> const> const B,
                  cublasHandle_t const handle, cudaStream_t const stream = nullptr,
                  cublasOperation_t const transA = CUBLAS_OP_N, cublasOperation_t const transB = CUBLAS_OP_N) {
        (void)handle;
        if (!A) throw std::invalid_argument("mpFlow::numeric::Matrix::multiply: A == nullptr");
        if (!B) throw std::invalid_argument("mpFlow::numeric::Matrix::multiply: B == nullptr");
        const bool ta = transA != CUBLAS_OP_N, tb = transB != CUBLAS_OP_N;
        const unsigned m = ta ? A->cols : A->rows, k = ta ? A->rows : A->cols;
        const unsigned kb = tb ? B->cols : B->rows, n = tb ? B->rows : B->cols;
        if (k != kb || m != rows || n != cols)
            throw std::invalid_argument("mpFlow::numeric::Matrix::multiply: shape does not match");
        detail::check(mpf_matrix_multiply(ta ? 1 : 0, tb ? 1 : 0, (int32_t)m, (int32_t)n, (int32_t)k, A->deviceData,
                                          (int32_t)A->dataRows, B->deviceData, (int32_t)B->dataRows, deviceData,
                                          (int32_t)dataRows, stream),
                      "mpFlow::numeric::Matrix::multiply");
    }
    // this = A B with a sparse A (src/numeric/matrix.cpp:335-349)
    template <template <class> class SparseType>
    void multiply(std::shared_ptr<SparseType<type> const> const A, std::shared_ptr<Matrix<type> const> const B,
                  cublasHandle_t const handle, cudaStream_t const stream = nullptr) {
        (void)handle;
        if (!A) throw std::invalid_argument("mpFlow::numeric::Matrix::multiply: A == nullptr");
        A->multiply(B, stream, std::shared_ptr<Matrix<type>>(this, [](Matrix<type>*) {}));
    }

    type& operator()(unsigned const i, unsigned const j) {
        requireHost("operator()");
        if (i >= rows || j >= cols) throw std::invalid_argument("mpFlow::numeric::Matrix::operator(): index out of range");
        return host_[i + (size_t)j * dataRows];
    }
    type operator()(unsigned const i, unsigned const j) const {
        requireHost("operator()");
        if (i >= rows || j >= cols) throw std::invalid_argument("mpFlow::numeric::Matrix::operator(): index out of range");
        return host_[i + (size_t)j * dataRows];
    }

    // text I/O (src/numeric/matrix.cpp:684-822): whitespace-separated rows
    static std::shared_ptr<Matrix<type>> loadtxt(std::istream& istream, cudaStream_t const stream = nullptr) {
        std::vector<std::vector<type>> values;
        std::string line;
        while (std::getline(istream, line)) {
            std::istringstream ls(line);
            std::vector<type> row;
            type v;
            while (ls >> v) row.push_back(v);
            if (!row.empty()) values.push_back(row);
        }
        if (values.empty()) throw std::runtime_error("mpFlow::numeric::Matrix::loadtxt: no values");
        auto m = std::make_shared<Matrix<type>>((unsigned)values.size(), (unsigned)values[0].size(), stream);
        for (unsigned i = 0; i < m->rows; ++i) {
            if (values[i].size() != m->cols) throw std::runtime_error("mpFlow::numeric::Matrix::loadtxt: ragged rows");
            for (unsigned j = 0; j < m->cols; ++j) (*m)(i, j) = values[i][j];
        }
        m->copyToDevice(stream);
        return m;
    }
    static std::shared_ptr<Matrix<type>> loadtxt(std::string const filename, cudaStream_t const stream = nullptr) {
        std::ifstream f(filename);
        if (!f) throw std::runtime_error("mpFlow::numeric::Matrix::loadtxt: cannot open file: " + filename);
        return loadtxt(f, stream);
    }
    // src/numeric/matrix.cpp:877-906: a JSON array of rows (or of values: one column)
    static std::shared_ptr<Matrix<type>> fromJsonArray(json::value const& array, cudaStream_t const stream = nullptr) {
        if (array.type != json::value::array || array.size() == 0) return nullptr;
        const unsigned rows = (unsigned)array.size();
        const unsigned cols = array[0].type == json::value::array ? (unsigned)array[0].size() : 1;
        auto m = std::make_shared<Matrix<type>>(rows, cols, stream);
        for (unsigned r = 0; r < rows; ++r)
            for (unsigned c = 0; c < cols; ++c)
                (*m)(r, c) = (type)(cols == 1 && array[r].type != json::value::array ? array[r].asDouble()
                                                                                    : array[r][c].asDouble());
        m->copyToDevice(stream);
        return m;
    }

    void savetxt(std::ostream& ostream) const {
        ostream << std::setprecision(std::numeric_limits<type>::max_digits10);
        for (unsigned i = 0; i < rows; ++i) {
            for (unsigned j = 0; j < cols; ++j) ostream << (j ? " " : "") << (*this)(i, j);
            ostream << "\n";
        }
    }
    void savetxt(std::string const filename) const {
        std::ofstream f(filename);
        if (!f) throw std::runtime_error("mpFlow::numeric::Matrix::savetxt: cannot open file: " + filename);
        savetxt(f);
    }

    unsigned const rows, cols, dataRows, dataCols;
    type* deviceData = nullptr;
    type* hostData() const { return host_.data(); }
    // the EIT model whose solve produced this matrix (used by solver::Inverse)
    mpf_eit_t owner = nullptr;

private:
    void requireHost(const char* what) const {
        if (host_.empty())
            throw std::logic_error(std::string("mpFlow::numeric::Matrix::") + what + ": host memory was not allocated");
    }
    void sameShape(std::shared_ptr<Matrix<type> const> const& other, const char* what) const {
        if (!other) throw std::invalid_argument(std::string("mpFlow::numeric::Matrix::") + what + ": matrix == nullptr");
        if (other->rows != rows || other->cols != cols || other->dataRows != dataRows)
            throw std::invalid_argument(std::string("mpFlow::numeric::Matrix::") + what + ": shape does not match");
    }
    void elementwise(int op, const type* A, const type* B, type scalar, cudaStream_t stream, const char* what) {
        detail::check(mpf_matrix_elementwise(op, (int32_t)rows, (int32_t)cols, A, B, deviceData, (int32_t)dataRows,
                                             (float)scalar, stream),
                      (std::string("mpFlow::numeric::Matrix::") + what).c_str());
    }
    void reduce(int op, std::shared_ptr<Matrix<type> const> const& A, const type* B, cudaStream_t stream,
                const char* what) {
        detail::check(mpf_matrix_column_reduce(op, (int32_t)rows, (int32_t)cols, A->deviceData, B, (int32_t)dataRows,
                                               deviceData, (int32_t)dataRows, stream),
                      (std::string("mpFlow::numeric::Matrix::") + what).c_str());
    }
    mutable std::vector<type> host_;
};

// Sparse matrix in the reference ELL layout (include/mpflow/numeric/
// sparse_matrix.h): dataRows x 32 values and column ids, row-major,
// 0xFFFFFFFF padding, host and device copies.  multiply() and the solvers
// below run in the library on its own copy (mpf_sparse_*), refreshed when
// the device arrays changed through copyToDevice().
template <class type_>
class SparseMatrix {
public:
    typedef type_ type;
    static unsigned const blockSize = 32;
    static unsigned const invalidIndex = 0xFFFFFFFFu;

    SparseMatrix(unsigned const rows, unsigned const cols, cudaStream_t const stream = nullptr)
        : rows(rows), cols(cols) {
        init(stream);
    }
    // src/numeric/sparse_matrix.cpp:29-42, 202-226: the nonzeros of every row
    // in column order (the matrix's host copy is read)
    SparseMatrix(std::shared_ptr<Matrix<type> const> const matrix, cudaStream_t const stream = nullptr)
        : rows(matrix ? matrix->rows : 0), cols(matrix ? matrix->cols : 0) {
        if (!matrix) throw std::invalid_argument("mpFlow::numeric::numeric::SparseMatrix::SparseMatrix: matrix == nullptr");
        init(stream);
        for (unsigned i = 0; i < rows; ++i)
            for (unsigned j = 0; j < cols; ++j)
                if ((*matrix)(i, j) != type(0)) setValue(i, j, (*matrix)(i, j));
        copyToDevice(stream);
    }
    SparseMatrix(SparseMatrix const&) = delete;
    SparseMatrix& operator=(SparseMatrix const&) = delete;
    virtual ~SparseMatrix() {
        if (handle_) mpf_sparse_destroy(handle_);
        cudaFree(deviceValues);
        cudaFree(deviceColumnIds);
    }

    void copyToDevice(cudaStream_t const stream = nullptr) {
        detail::cuda(cudaMemcpyAsync(deviceValues, hostValues_.data(), sizeof(type) * hostValues_.size(),
                                     cudaMemcpyHostToDevice, stream),
                     "mpFlow::numeric::SparseMatrix::copyToDevice");
        detail::cuda(cudaMemcpyAsync(deviceColumnIds, hostColumnIds_.data(), sizeof(unsigned) * hostColumnIds_.size(),
                                     cudaMemcpyHostToDevice, stream),
                     "mpFlow::numeric::SparseMatrix::copyToDevice");
        detail::cuda(cudaStreamSynchronize(stream), "mpFlow::numeric::SparseMatrix::copyToDevice");
        dirty_ = true;
    }
    void copyToHost(cudaStream_t const stream = nullptr) {
        detail::cuda(cudaMemcpyAsync(hostValues_.data(), deviceValues, sizeof(type) * hostValues_.size(),
                                     cudaMemcpyDeviceToHost, stream),
                     "mpFlow::numeric::SparseMatrix::copyToHost");
        detail::cuda(cudaMemcpyAsync(hostColumnIds_.data(), deviceColumnIds, sizeof(unsigned) * hostColumnIds_.size(),
                                     cudaMemcpyDeviceToHost, stream),
                     "mpFlow::numeric::SparseMatrix::copyToHost");
        detail::cuda(cudaStreamSynchronize(stream), "mpFlow::numeric::SparseMatrix::copyToHost");
    }

    // src/numeric/sparse_matrix.cpp:358-423 (host arrays)
    unsigned getColumnId(unsigned const row, unsigned const col) const {
        return hostColumnIds_[(size_t)row * blockSize + col];
    }
    type getValue(unsigned const row, unsigned const col) const {
        for (unsigned i = 0; i < blockSize; ++i)
            if (hostColumnIds_[(size_t)row * blockSize + i] == col) return hostValues_[(size_t)row * blockSize + i];
        return type(0);
    }
    void setValue(unsigned const row, unsigned const col, type const& value) {
        if (row >= rows || col >= cols)
            throw std::logic_error("mpFlow::numeric::SparseMatrix::setValue(): index out of range");
        unsigned slot = invalidIndex;
        for (unsigned i = 0; i < blockSize; ++i) {
            unsigned& id = hostColumnIds_[(size_t)row * blockSize + i];
            if (id == col) {
                slot = i;
                break;
            }
            if (id == invalidIndex) {
                slot = i;
                id = col;
                density = std::max(density, i + 1);
                break;
            }
        }
        if (slot == invalidIndex) throw std::logic_error("mpFlow::numeric::SparseMatrix::operator(): sparse format full");
        hostValues_[(size_t)row * blockSize + slot] = value;
    }

    // src/numeric/sparse_matrix.cpp:262-288: result = this * matrix (device data)
    void multiply(std::shared_ptr<Matrix<type> const> const matrix, cudaStream_t const stream,
                  std::shared_ptr<Matrix<type>> result) const {
        if (!matrix) throw std::invalid_argument("mpFlow::numeric::SparseMatrix::multiply: matrix == nullptr");
        if (!result) throw std::invalid_argument("mpFlow::numeric::SparseMatrix::multiply: result == nullptr");
        if (matrix->rows != cols || result->rows != rows || result->cols != matrix->cols)
            throw std::invalid_argument("mpFlow::numeric::SparseMatrix::multiply: shape does not match");
        detail::check(mpf_sparse_multiply(handle(), matrix->deviceData, (int32_t)matrix->dataRows,
                                          (int32_t)matrix->cols, result->deviceData, (int32_t)result->dataRows,
                                          stream),
                      "mpFlow::numeric::SparseMatrix::multiply");
    }

    // src/numeric/sparse_matrix.cpp:228-244 (host copy)
    std::shared_ptr<Matrix<type>> toMatrix(cudaStream_t const stream = nullptr) const {
        auto m = std::make_shared<Matrix<type>>(rows, cols, stream);
        for (unsigned i = 0; i < rows; ++i)
            for (unsigned k = 0; k < blockSize; ++k) {
                const unsigned c = hostColumnIds_[(size_t)i * blockSize + k];
                if (c != invalidIndex) (*m)(i, c) = hostValues_[(size_t)i * blockSize + k];
            }
        m->copyToDevice(stream);
        return m;
    }

    // the library's copy of the device arrays
    mpf_sparse_t handle() const {
        if (dirty_ || !handle_) {
            if (handle_) mpf_sparse_destroy(handle_);
            handle_ = nullptr;
            detail::check(mpf_sparse_create((int32_t)rows, deviceValues, deviceColumnIds, density, &handle_),
                          "mpFlow::numeric::SparseMatrix");
            dirty_ = false;
        }
        return handle_;
    }

    unsigned const rows;
    unsigned const cols;
    unsigned dataRows = 0;
    unsigned dataCols = 0;
    unsigned density = 0;
    type* deviceValues = nullptr;
    unsigned* deviceColumnIds = nullptr;

private:
    void init(cudaStream_t const stream) {
        if (rows == 0) throw std::invalid_argument("mpFlow::numeric::numeric::SparseMatrix::init: rows == 0");
        if (cols == 0) throw std::invalid_argument("mpFlow::numeric::numeric::SparseMatrix::init: columns == 0");
        dataRows = mpf_data_rows(rows);
        dataCols = mpf_data_rows(cols);
        hostValues_.assign((size_t)dataRows * blockSize, type(0));
        hostColumnIds_.assign((size_t)dataRows * blockSize, invalidIndex);
        detail::cuda(cudaMalloc((void**)&deviceValues, sizeof(type) * hostValues_.size()),
                     "mpFlow::numeric::SparseMatrix::init: create device data memory");
        detail::cuda(cudaMalloc((void**)&deviceColumnIds, sizeof(unsigned) * hostColumnIds_.size()),
                     "mpFlow::numeric::SparseMatrix::init: create device data memory");
        copyToDevice(stream);
    }
    std::vector<type> hostValues_;
    std::vector<unsigned> hostColumnIds_;
    mutable mpf_sparse_t handle_ = nullptr;
    mutable bool dirty_ = true;
};

// numeric::preconditioner::diagonal (src/numeric/preconditioner.cpp:23-76,
// kernels src/numeric/preconditioner_kernel.cu:31-83): result = D^-1 as a
// 1-slot sparse matrix (slot 0 column = row, value 1 / a_ii; the dense form
// divides by a_ii as the reference does, the sparse form leaves 0 where the
// row has no diagonal entry).  Computed on the host copies; the solvers of
// this library apply the same Jacobi preconditioner internally.
namespace preconditioner {
template <class type>
void diagonal(std::shared_ptr<Matrix<type> const> const matrix, cudaStream_t const stream,
              std::shared_ptr<SparseMatrix<type>> const result) {
    if (!matrix) throw std::invalid_argument("mpFlow::numeric::preconditioner::diagonal: matrix == nullptr");
    if (!result) throw std::invalid_argument("mpFlow::numeric::preconditioner::diagonal: result == nullptr");
    const_cast<Matrix<type>&>(*matrix).copyToHost(stream);
    for (unsigned i = 0; i < matrix->rows && i < result->rows; ++i) result->setValue(i, i, type(1) / (*matrix)(i, i));
    result->density = 1;
    result->copyToDevice(stream);
}
template <class type>
void diagonal(std::shared_ptr<SparseMatrix<type> const> const matrix, cudaStream_t const stream,
              std::shared_ptr<SparseMatrix<type>> const result) {
    if (!matrix) throw std::invalid_argument("mpFlow::numeric::preconditioner::diagonal: matrix == nullptr");
    if (!result) throw std::invalid_argument("mpFlow::numeric::preconditioner::diagonal: result == nullptr");
    for (unsigned i = 0; i < matrix->rows && i < result->rows; ++i) {
        const type d = matrix->getValue(i, i);
        result->setValue(i, i, d != type(0) ? type(1) / d : type(0));
    }
    result->density = 1;
    result->copyToDevice(stream);
}
}  // namespace preconditioner

namespace krylov {
// numeric::ConjugateGradient / numeric::BiCGSTAB solve through mpf_sparse_solve
template <class dataType>
unsigned solve(int32_t solver, std::shared_ptr<SparseMatrix<dataType>> const A,
                      std::shared_ptr<Matrix<dataType> const> const b, cudaStream_t const stream,
                      std::shared_ptr<Matrix<dataType>> const x, unsigned const maxIterations, bool const dcFree,
                      char const* where) {
    if (!A) throw std::invalid_argument(std::string(where) + ": A == nullptr");
    if (!b) throw std::invalid_argument(std::string(where) + ": b == nullptr");
    if (!x) throw std::invalid_argument(std::string(where) + ": x == nullptr");
    int32_t iterations = 0;
    const int status = mpf_sparse_solve(A->handle(), solver, b->deviceData, (int32_t)b->dataRows, x->deviceData,
                                        (int32_t)x->dataRows, (int32_t)b->cols, (int32_t)maxIterations, 0.0,
                                        dcFree ? 1 : 0, &iterations, stream);
    if (status != MPF_OK && status != MPF_ENOCONV) mpFlow::detail::check(status, where);
    return (unsigned)iterations;
}
}  // namespace krylov

// numeric::ConjugateGradient (include/mpflow/numeric/conjugate_gradient.h):
// all columns of b at once, Jacobi-preconditioned (KInv is accepted and
// the diagonal preconditioner used in its place), the reference's
// stopping level and iteration cap; returns the iterations of the slowest
// column.  Also the solver tag of models::EIT.
template <class dataType>
class ConjugateGradient {
public:
    ConjugateGradient(unsigned const rows, unsigned const cols, cudaStream_t const stream = nullptr)
        : rows(rows), cols(cols) {
        (void)stream;
        if (rows < 1) throw std::invalid_argument("mpFlow::numeric::ConjugateGradient::ConjugateGradient: rows <= 1");
        if (cols < 1) throw std::invalid_argument("mpFlow::numeric::ConjugateGradient::ConjugateGradient: cols <= 1");
    }
    template <template <class> class matrixType, template <class> class preconditionerType = matrixType>
    unsigned solve(std::shared_ptr<matrixType<dataType>> const A, std::shared_ptr<Matrix<dataType> const> const b,
                   cublasHandle_t const handle, cudaStream_t const stream, std::shared_ptr<Matrix<dataType>> const x,
                   std::shared_ptr<preconditionerType<dataType>> const KInv = nullptr, unsigned const maxIterations = 0,
                   bool const dcFree = false) {
        (void)handle;
        (void)KInv;
        return krylov::solve(0, A, b, stream, x, maxIterations, dcFree, "mpFlow::numeric::ConjugateGradient::solve");
    }
    unsigned const rows;
    unsigned const cols;
};

// numeric::BiCGSTAB (include/mpflow/numeric/bicgstab.h), as above
template <class dataType>
class BiCGSTAB {
public:
    BiCGSTAB(unsigned const rows, unsigned const cols, cudaStream_t const stream = nullptr) : rows(rows), cols(cols) {
        (void)stream;
        if (rows < 1) throw std::invalid_argument("mpFlow::numeric::BiCGSTAB::BiCGSTAB: rows <= 1");
        if (cols < 1) throw std::invalid_argument("mpFlow::numeric::BiCGSTAB::BiCGSTAB: cols <= 1");
    }
    template <template <class> class matrixType, template <class> class preconditionerType = matrixType>
    unsigned solve(std::shared_ptr<matrixType<dataType>> const A, std::shared_ptr<Matrix<dataType> const> const b,
                   cublasHandle_t const handle, cudaStream_t const stream, std::shared_ptr<Matrix<dataType>> const x,
                   std::shared_ptr<preconditionerType<dataType>> const KInv = nullptr, unsigned const maxIterations = 0,
                   bool const dcFree = false) {
        (void)handle;
        (void)KInv;
        return krylov::solve(1, A, b, stream, x, maxIterations, dcFree, "mpFlow::numeric::BiCGSTAB::solve");
    }
    unsigned const rows;
    unsigned const cols;
};

// mpf_solve_opts::solver of a solver tag
template <template <class> class S>
struct SolverCode {
    static int32_t const value = 0;
};
template <>
struct SolverCode<BiCGSTAB> {
    static int32_t const value = 1;
};

// Triangular mesh (src/numeric/irregular_mesh.cpp); edges, element edges and
// boundary are derived by mpf_mesh_edges.
class IrregularMesh {
public:
    IrregularMesh(Array2<double> const& nodes, Array2<int> const& elements) : nodes(nodes), elements(elements) {
        if (nodes.cols() != 2) throw std::invalid_argument("mpFlow::numeric::IrregularMesh::IrregularMesh: nodes.cols != 2");
        if (elements.cols() != 3)
            throw std::invalid_argument("mpFlow::numeric::IrregularMesh::IrregularMesh: elements.cols != 3");
        const unsigned e = elements.rows();
        std::vector<int32_t> ed((size_t)6 * e), ee((size_t)3 * e), bd((size_t)3 * e);
        int32_t ne = 0, nb = 0;
        detail::check(mpf_mesh_edges((int32_t)nodes.rows(), (int32_t)e, nodes.data.data(), elements.data.data(),
                                     ed.data(), ee.data(), bd.data(), &ne, &nb),
                      "mpFlow::numeric::IrregularMesh::IrregularMesh");
        edges = Array2<int>((unsigned)ne, 2);
        std::copy(ed.begin(), ed.begin() + 2 * (size_t)ne, edges.data.begin());
        elementEdges = Array2<int>(e, 3);
        std::copy(ee.begin(), ee.end(), elementEdges.data.begin());
        boundary.assign(bd.begin(), bd.begin() + nb);
    }

    // concentric-ring disk (stands in for the distmesh branch of fromConfig)
    static std::shared_ptr<IrregularMesh> ring(unsigned const rings, double const radius = 1.0) {
        int32_t n = 0, e = 0;
        detail::check(mpf_ring_mesh_counts((int32_t)rings, &n, &e), "mpFlow::numeric::IrregularMesh::ring");
        Array2<double> nd((unsigned)n, 2);
        Array2<int> el((unsigned)e, 3);
        detail::check(mpf_ring_mesh((int32_t)rings, radius, nd.data.data(), el.data.data()),
                      "mpFlow::numeric::IrregularMesh::ring");
        return std::make_shared<IrregularMesh>(nd, el);
    }

    // src/numeric/irregular_mesh.cpp:48-126: a mesh directory (string, or
    // {"path": ...}) holding nodes.txt and elements.txt; edges are always
    // derived here.  The reference's distmesh branch ({"radius",
    // "outerEdgeLength", "innerEdgeLength"}) needs libdistmesh, which this
    // library does not carry; {"rings": R, "radius": r} builds the ring mesh.
    static std::shared_ptr<IrregularMesh> fromConfig(json::value const& config, json::value const& portConfig,
                                                     cudaStream_t const stream, std::string const path = "./") {
        (void)portConfig;
        if (config.type == json::value::string || config["path"].type == json::value::string) {
            const std::string dir = path + "/" + (config.type == json::value::string ? config.str : config["path"].str);
            auto nodes = Matrix<double>::loadtxt(dir + "/nodes.txt", stream);
            auto elements = Matrix<int>::loadtxt(dir + "/elements.txt", stream);
            Array2<double> nd(nodes->rows, nodes->cols);
            for (unsigned i = 0; i < nodes->rows; ++i)
                for (unsigned j = 0; j < nodes->cols; ++j) nd(i, j) = (*nodes)(i, j);
            Array2<int> el(elements->rows, elements->cols);
            for (unsigned i = 0; i < elements->rows; ++i)
                for (unsigned j = 0; j < elements->cols; ++j) el(i, j) = (*elements)(i, j);
            return std::make_shared<IrregularMesh>(nd, el);
        }
        if (config["rings"].type == json::value::number)
            return ring((unsigned)config["rings"].asInt(), config["radius"].asDouble(1.0));
        if (config["outerEdgeLength"].type != json::value::none)
            throw std::runtime_error(
                "mpFlow::numeric::IrregularMesh::fromConfig: distmesh meshing is not available; give a mesh "
                "directory or {\"rings\": R, \"radius\": r}");
        return nullptr;
    }

    Array2<double> elementNodes(unsigned const element) const {
        Array2<double> out(3, 2);
        for (unsigned i = 0; i < 3; ++i)
            for (unsigned k = 0; k < 2; ++k) out(i, k) = nodes(elements(element, i), k);
        return out;
    }
    Array2<double> edgeNodes(unsigned const edge) const {
        Array2<double> out(2, 2);
        for (unsigned i = 0; i < 2; ++i)
            for (unsigned k = 0; k < 2; ++k) out(i, k) = nodes(edges(edge, i), k);
        return out;
    }

    Array2<double> const nodes;
    Array2<int> const elements;
    Array2<int> elementEdges;
    Array2<int> edges;
    std::vector<int> boundary;
};

}  // namespace numeric

namespace FEM {

namespace basis {
class Linear {};
}  // namespace basis

// equation template tag: data type, basis, logarithmic parametrisation
template <class dataType_ = float, class basisFunctionType = basis::Linear, bool logarithmic_ = true>
class Equation {
public:
    typedef dataType_ dataType;
    static bool const logarithmic = logarithmic_;
};

class Ports {
public:
    explicit Ports(numeric::Array2<int> const& edges) : edges(edges), count(edges.rows()) {
        if (edges.rows() == 0) throw std::invalid_argument("mpFlow::FEM::Ports::Ports: edges.rows() == 0");
    }
    virtual ~Ports() {}

    static std::shared_ptr<Ports> circularBoundary(unsigned const count, double const width,
                                                   std::shared_ptr<numeric::IrregularMesh const> const mesh,
                                                   double const offset = 0.0, bool const clockwise = false) {
        if (!mesh) throw std::invalid_argument("mpFlow::FEM::Ports::circularBoundary: mesh == nullptr");
        const int32_t cap = 512;
        std::vector<int32_t> out((size_t)count * cap, -1);
        int32_t mx = 0;
        detail::check(mpf_ports_circular((int32_t)mesh->nodes.rows(), mesh->nodes.data.data(),
                                         (int32_t)mesh->elements.rows(), mesh->elements.data.data(),
                                         mesh->edges.data.data(), (int32_t)mesh->boundary.size(),
                                         mesh->boundary.data(), (int32_t)count, width, offset, clockwise ? 1 : 0,
                                         out.data(), cap, &mx),
                      "mpFlow::FEM::Ports::circularBoundary");
        numeric::Array2<int> e(count, (unsigned)std::max(mx, 1), -1);
        for (unsigned p = 0; p < count; ++p)
            for (unsigned k = 0; k < e.cols(); ++k) e(p, k) = out[(size_t)p * cap + k];
        return std::make_shared<Ports>(e);
    }

    // src/fem/ports.cpp:79-114: a file of port edges (string or {"edges":
    // file}) or {"count", "width", "offset", "clockwise"} on a circular boundary
    static std::shared_ptr<Ports> fromConfig(json::value const& config,
                                             std::shared_ptr<numeric::IrregularMesh const> const mesh,
                                             cudaStream_t const stream, std::string const path = "./",
                                             std::string const meshPath = "./mesh") {
        (void)meshPath;
        if (config.type == json::value::string || config["edges"].type == json::value::string) {
            auto m = numeric::Matrix<int>::loadtxt(
                path + "/" + (config.type == json::value::string ? config.str : config["edges"].str), stream);
            numeric::Array2<int> e(m->rows, m->cols);
            for (unsigned i = 0; i < m->rows; ++i)
                for (unsigned j = 0; j < m->cols; ++j) e(i, j) = (*m)(i, j);
            return std::make_shared<Ports>(e);
        }
        return circularBoundary((unsigned)config["count"].asInt(), config["width"].asDouble(),
                                mesh, config["offset"].asDouble(), config["clockwise"].asBool());
    }

    numeric::Array2<int> const edges;
    unsigned const count;
};

template <class dataType>
class Sources {
public:
    enum Type { Open, Fixed };

    Sources(Type const type, std::vector<dataType> const& values, std::shared_ptr<Ports const> const ports,
            std::shared_ptr<numeric::Matrix<int> const> const drivePattern,
            std::shared_ptr<numeric::Matrix<int> const> const measurementPattern, cudaStream_t const stream)
        : type(type), values(values), ports(ports) {
        if (!ports) throw std::invalid_argument("mpFlow::FEM::Sources::Sources: ports == nullptr");
        if (!drivePattern) throw std::invalid_argument("mpFlow::FEM::Sources::Sources: drivePattern == nullptr");
        if (!measurementPattern)
            throw std::invalid_argument("mpFlow::FEM::Sources::Sources: measurementPattern == nullptr");
        if (values.size() != drivePattern->cols)
            throw std::invalid_argument("mpFlow::FEM::Sources::Sources: invalid size of values vector");
        this->drivePattern = convert(drivePattern, stream);
        this->measurementPattern = convert(measurementPattern, stream);
        // pattern = [value_c * drive_c | meas] (src/fem/sources.cpp:50-75)
        const unsigned L = drivePattern->rows, Md = drivePattern->cols, Mm = measurementPattern->cols;
        pattern = std::make_shared<numeric::Matrix<dataType>>(L, Md + Mm, stream);
        for (unsigned i = 0; i < L; ++i) {
            for (unsigned j = 0; j < Md; ++j) (*pattern)(i, j) = values[j] * (dataType)(*drivePattern)(i, j);
            for (unsigned j = 0; j < Mm; ++j) (*pattern)(i, Md + j) = (dataType)(*measurementPattern)(i, j);
        }
        pattern->copyToDevice(stream);
    }
    Sources(Type const type, dataType const value, std::shared_ptr<Ports const> const ports,
            std::shared_ptr<numeric::Matrix<int> const> const drivePattern,
            std::shared_ptr<numeric::Matrix<int> const> const measurementPattern, cudaStream_t const stream)
        : Sources(type, std::vector<dataType>(drivePattern ? drivePattern->cols : 0, value), ports, drivePattern,
                  measurementPattern, stream) {}
    virtual ~Sources() {}

    // src/fem/sources.cpp:92-131: "type" ("voltage" -> Fixed, else Open),
    // "value" (number or per-pattern array, default 1), "drivePattern" and
    // "measurementPattern" as JSON arrays of rows (default: identity)
    static std::shared_ptr<Sources<dataType>> fromConfig(json::value const& config, std::shared_ptr<Ports const> const ports,
                                                         cudaStream_t const stream) {
        auto pattern = [&](json::value const& c) {
            auto m = numeric::Matrix<int>::fromJsonArray(c, stream);
            return m ? m : numeric::Matrix<int>::eye(ports->count, stream);
        };
        auto drive = pattern(config["drivePattern"]);
        auto meas = pattern(config["measurementPattern"]);
        std::vector<dataType> excitation(drive->cols);
        for (unsigned i = 0; i < drive->cols; ++i)
            excitation[i] = (dataType)(config["value"].type == json::value::array ? config["value"][i].asDouble()
                                                                                  : config["value"].asDouble(1.0));
        const Type t = config["type"].asString() == "voltage" ? Fixed : Open;
        return std::make_shared<Sources<dataType>>(t, excitation, ports, drive, meas, stream);
    }

    Type const type;
    std::vector<dataType> const values;
    std::shared_ptr<Ports const> const ports;
    std::shared_ptr<numeric::Matrix<dataType>> drivePattern;
    std::shared_ptr<numeric::Matrix<dataType>> measurementPattern;
    std::shared_ptr<numeric::Matrix<dataType>> pattern;

private:
    static std::shared_ptr<numeric::Matrix<dataType>> convert(std::shared_ptr<numeric::Matrix<int> const> const m,
                                                              cudaStream_t const stream) {
        auto out = std::make_shared<numeric::Matrix<dataType>>(m->rows, m->cols, stream);
        for (unsigned i = 0; i < m->rows; ++i)
            for (unsigned j = 0; j < m->cols; ++j) (*out)(i, j) = (dataType)(*m)(i, j);
        out->copyToDevice(stream);
        return out;
    }
};

}  // namespace FEM

namespace models {

// 2.5D EIT forward model (src/models/eit.cpp).  Besides the reference's
// members it carries `options` (mpf_solve_opts: tolerance, refinement,
// preconditioner) and `handle()` for direct C-ABI calls.
template <template <class> class numericalSolverType = numeric::ConjugateGradient,
          class equationType_ = FEM::Equation<float, FEM::basis::Linear, false>>
class EIT {
public:
    typedef equationType_ equationType;
    typedef typename equationType::dataType dataType;
    static bool const logarithmic = equationType::logarithmic;

    EIT(std::shared_ptr<numeric::IrregularMesh const> const mesh, std::shared_ptr<FEM::Sources<dataType> const> const sources,
        dataType const referenceValue, cublasHandle_t const handle, cudaStream_t const stream,
        unsigned const components = 1, double const height = 1.0, double const portHeight = 1.0)
        : mesh(mesh), sources(sources), referenceValue(referenceValue), height(height), portHeight(portHeight) {
        (void)handle;
        if (!mesh) throw std::invalid_argument("mpFlow::models::EIT::EIT: mesh == nullptr");
        if (!sources) throw std::invalid_argument("mpFlow::models::EIT::EIT: sources == nullptr");
        const unsigned L = sources->ports->count, Md = sources->drivePattern->cols, Mm = sources->measurementPattern->cols;
        std::vector<double> drive((size_t)L * Md), meas((size_t)L * Mm), vals;
        for (auto const& v : sources->values) vals.push_back(detail::real_part(v));
        for (unsigned j = 0; j < Md; ++j)
            for (unsigned i = 0; i < L; ++i) drive[i + (size_t)j * L] = detail::real_part((*sources->drivePattern)(i, j));
        for (unsigned j = 0; j < Mm; ++j)
            for (unsigned i = 0; i < L; ++i) meas[i + (size_t)j * L] = detail::real_part((*sources->measurementPattern)(i, j));
        // complex models (thrust::complex instantiations, src/models/eit.cpp:289-304):
        // currents and the reference value are real; a complex admittivity
        // is expressed through the material distribution
        if (detail::imag_part(referenceValue) != 0.0)
            throw std::invalid_argument("mpFlow::models::EIT::EIT: complex referenceValue (express it through the "
                                        "material distribution)");
        for (auto const& v : sources->values)
            if (detail::imag_part(v) != 0.0)
                throw std::invalid_argument("mpFlow::models::EIT::EIT: complex source values are not supported");
        int device = 0;
        detail::cuda(cudaGetDevice(&device), "mpFlow::models::EIT::EIT");
        mpf_eit_desc d{};
        d.n_nodes = (int32_t)mesh->nodes.rows();
        d.n_elements = (int32_t)mesh->elements.rows();
        d.nodes = mesh->nodes.data.data();
        d.elements = mesh->elements.data.data();
        d.edges = mesh->edges.data.data();
        d.n_edges = (int32_t)mesh->edges.rows();
        d.ports = (int32_t)L;
        d.port_edges = sources->ports->edges.data.data();
        d.port_edges_cap = (int32_t)sources->ports->edges.cols();
        d.drive_count = (int32_t)Md;
        d.meas_count = (int32_t)Mm;
        d.drive_pattern = drive.data();
        d.meas_pattern = meas.data();
        d.source_values = vals.data();
        d.source_type = sources->type == FEM::Sources<dataType>::Open ? MPF_SOURCE_OPEN : MPF_SOURCE_FIXED;
        d.reference_value = detail::real_part(referenceValue);
        d.logarithmic = logarithmic ? 1 : 0;
        d.components = (int32_t)components;
        d.height = height;
        d.port_height = portHeight;
        d.device = device;
        d.jacobian_mode = 0;
        detail::check(mpf_eit_create(&d, &model_), "mpFlow::models::EIT::EIT");
        detail::check(mpf_eit_get_info(model_, &info_), "mpFlow::models::EIT::EIT");
        result = std::make_shared<numeric::Matrix<dataType>>(Mm, Md, stream);
        jacobian = std::make_shared<numeric::Matrix<dataType>>((unsigned)info_.jacobian_rows, mesh->elements.rows(), stream,
                                                               dataType(0), false);
        jacobian->owner = model_;
        result->owner = model_;
        for (unsigned c = 0; c < components; ++c)
            fields.push_back(std::make_shared<numeric::Matrix<dataType>>(mesh->nodes.rows(), Md + Mm, stream,
                                                                         dataType(0), false));
        field = fields[0];
        options.tol = 1e-6;
        options.max_iter = 0;
        options.refine_tol = 0.0;
        options.max_refine = 6;
        options.warm_start = 0;
        options.check_every = 16;
        options.preconditioner = 0;
        options.solver = numeric::SolverCode<numericalSolverType>::value;
    }
    EIT(EIT const&) = delete;
    EIT& operator=(EIT const&) = delete;
    virtual ~EIT() { mpf_eit_destroy(model_); }

    // src/models/eit.cpp:102-131
    static std::shared_ptr<EIT<numericalSolverType, equationType>> fromConfig(
        json::value const& config, cublasHandle_t const handle, cudaStream_t const stream, std::string const path = "./",
        std::shared_ptr<numeric::IrregularMesh const> const externalMesh = nullptr) {
        auto const mesh = externalMesh ? externalMesh
                                       : std::shared_ptr<numeric::IrregularMesh const>(
                                             numeric::IrregularMesh::fromConfig(config["mesh"], config["ports"], stream, path));
        if (!mesh) throw std::invalid_argument("mpFlow::models::EIT::fromConfig: invalid mesh config");
        const std::string meshPath = config["mesh"].type == json::value::string ? config["mesh"].str
                                     : config["mesh"]["path"].type == json::value::string ? config["mesh"]["path"].str
                                                                                           : std::string("mesh");
        auto const ports = FEM::Ports::fromConfig(config["ports"], mesh, stream, path, meshPath);
        auto const sources = FEM::Sources<dataType>::fromConfig(config["source"], ports, stream);
        const dataType referenceValue = (dataType)(config["material"].type == json::value::object
                                                       ? config["material"]["referenceValue"].asDouble(1.0)
                                                       : config["material"].asDouble(1.0));
        const unsigned components = (unsigned)std::max(1L, config["2.5D"]["components"].asInt(1));
        const double height = config["2.5D"]["height"].asDouble(1.0);
        const double portHeight = config["ports"]["height"].asDouble(1.0);
        return std::make_shared<EIT<numericalSolverType, equationType>>(mesh, sources, referenceValue, handle, stream,
                                                                        components, height, portHeight);
    }

    // forward solve of one material distribution (E x 1); returns the
    // Mm x Md electrode voltages and updates jacobian and fields
    std::shared_ptr<numeric::Matrix<dataType> const> solve(
        std::shared_ptr<numeric::Matrix<dataType> const> const materialDistribution, cublasHandle_t const handle,
        cudaStream_t const stream, unsigned* const steps = nullptr) {
        (void)handle;
        if (!materialDistribution)
            throw std::invalid_argument("mpFlow::models::EIT::solve: materialDistribution == nullptr");
        if (materialDistribution->rows != mesh->elements.rows())
            throw std::invalid_argument("mpFlow::models::EIT::solve: materialDistribution has wrong size");
        mpf_solve_stats st{};
        int status;
        if constexpr (detail::lib_native<dataType>()) {
            // float, thrust::complex<float>, std::complex<float>: the library's own precision
            const unsigned Mm = result->rows, Md = result->cols;
            dataType* V = nullptr;
            detail::cuda(cudaMallocAsync((void**)&V, sizeof(dataType) * (size_t)Mm * Md, stream),
                         "mpFlow::models::EIT::solve");
            if constexpr (detail::is_complex<dataType>::value) {
                // complex admittivity: complex BiCGSTAB whatever the solver tag
                // (the reference's CG on complex data is the same Krylov family)
                mpf_solve_opts o = options;
                o.solver = 1;
                status = mpf_eit_forward_complex(model_, 1,
                                                 reinterpret_cast<const float*>(materialDistribution->deviceData),
                                                 reinterpret_cast<float*>(V),
                                                 reinterpret_cast<float*>(jacobian->deviceData), &o, &st, stream);
            } else {
                status = mpf_eit_forward(model_, 1, materialDistribution->deviceData, V, jacobian->deviceData,
                                         &options, &st, stream);
            }
            if (status == MPF_OK || status == MPF_ENOCONV) {
                detail::cuda(cudaMemcpy2DAsync(result->deviceData, sizeof(dataType) * result->dataRows, V,
                                               sizeof(dataType) * Mm, sizeof(dataType) * Mm, Md,
                                               cudaMemcpyDeviceToDevice, stream),
                             "mpFlow::models::EIT::solve");
                fieldsValid_ = true;
            }
            cudaFreeAsync(V, stream);
        } else {
            status = solve_converted(materialDistribution, stream, &st);
        }
        detail::check(status == MPF_ENOCONV ? MPF_OK : status, "mpFlow::models::EIT::solve");
        detail::cuda(cudaStreamSynchronize(stream), "mpFlow::models::EIT::solve");
        if (steps) *steps = (unsigned)st.iterations;
        lastStats = st;
        return result;
    }

    // potentials of the last solve, one matrix per 2.5D component (complex
    // for the complex instantiations)
    void updateFields(cudaStream_t const stream) {
        if (!fieldsValid_) throw std::logic_error("mpFlow::models::EIT::updateFields: no solve yet");
        typedef detail::lib_type<dataType> L;
        const size_t per = (size_t)fields[0]->dataRows * fields[0]->cols;  // export layout: dataRows x cols per component
        L* buf = nullptr;
        detail::cuda(cudaMallocAsync((void**)&buf, sizeof(L) * per * fields.size(), stream), "updateFields");
        int st;
        if constexpr (detail::is_complex<dataType>::value)
            st = mpf_eit_fields_complex(model_, 1, reinterpret_cast<float*>(buf), stream);
        else
            st = mpf_eit_fields(model_, 1, buf, stream);
        if (st == MPF_OK)
            for (size_t c = 0; c < fields.size(); ++c)  // double / complex<double>: from the FP32 potentials
                detail::convert_device(fields[c]->deviceData, buf + c * per, per, stream,
                                       "mpFlow::models::EIT::updateFields");
        cudaFreeAsync(buf, stream);
        detail::check(st, "mpFlow::models::EIT::updateFields");
        detail::cuda(cudaStreamSynchronize(stream), "updateFields");
    }

    // jacobian *= mask (elementwise, same shape): Matrix::elementwiseMultiply
    // as the reference's noSensitivity option uses it (src/solver/solver.cpp:116-122)
    void maskJacobian(std::shared_ptr<numeric::Matrix<dataType> const> const mask, cudaStream_t const stream) {
        if (!mask || mask->rows != jacobian->rows || mask->cols != jacobian->cols)
            throw std::invalid_argument("mpFlow::models::EIT::maskJacobian: mask shape differs from the jacobian");
        const size_t n = (size_t)jacobian->dataRows * jacobian->cols;
        std::vector<dataType> J(n);
        detail::cuda(cudaMemcpyAsync(J.data(), jacobian->deviceData, sizeof(dataType) * n, cudaMemcpyDeviceToHost, stream),
                     "maskJacobian");
        detail::cuda(cudaStreamSynchronize(stream), "maskJacobian");
        for (unsigned j = 0; j < jacobian->cols; ++j)
            for (unsigned i = 0; i < jacobian->rows; ++i) J[i + (size_t)j * jacobian->dataRows] *= (*mask)(i, j);
        detail::cuda(cudaMemcpyAsync(jacobian->deviceData, J.data(), sizeof(dataType) * n, cudaMemcpyHostToDevice, stream),
                     "maskJacobian");
        detail::cuda(cudaStreamSynchronize(stream), "maskJacobian");
    }

    mpf_eit_t handle() const { return model_; }
    mpf_eit_info const& info() const { return info_; }

    std::shared_ptr<numeric::IrregularMesh const> const mesh;
    std::shared_ptr<FEM::Sources<dataType> const> const sources;
    dataType const referenceValue;
    double const height;
    double const portHeight;
    std::vector<std::shared_ptr<numeric::Matrix<dataType>>> fields;
    std::shared_ptr<numeric::Matrix<dataType>> field;
    std::shared_ptr<numeric::Matrix<dataType>> result;
    std::shared_ptr<numeric::Matrix<dataType>> jacobian;
    mpf_solve_opts options{};
    mpf_solve_stats lastStats{};

private:
    // double, complex<double>: through the library's FP32 interface, values
    // converted on the way in (material) and out (voltages, Jacobian)
    int solve_converted(std::shared_ptr<numeric::Matrix<dataType> const> const& materialDistribution,
                        cudaStream_t const stream, mpf_solve_stats* st) {
        typedef detail::lib_type<dataType> L;
        const char* where = "mpFlow::models::EIT::solve";
        const unsigned Mm = result->rows, Md = result->cols;
        const size_t E = mesh->elements.rows(), nJ = (size_t)jacobian->dataRows * E;
        L *V = nullptr, *g = nullptr, *Jl = nullptr;
        detail::cuda(cudaMallocAsync((void**)&V, sizeof(L) * (size_t)Mm * Md, stream), where);
        detail::cuda(cudaMallocAsync((void**)&g, sizeof(L) * E, stream), where);
        detail::cuda(cudaMallocAsync((void**)&Jl, sizeof(L) * nJ, stream), where);
        detail::convert_device(g, materialDistribution->deviceData, E, stream, where);
        int status;
        if constexpr (detail::is_complex<dataType>::value) {
            mpf_solve_opts o = options;
            o.solver = 1;
            status = mpf_eit_forward_complex(model_, 1, reinterpret_cast<const float*>(g), reinterpret_cast<float*>(V),
                                             reinterpret_cast<float*>(Jl), &o, st, stream);
        } else {
            status = mpf_eit_forward(model_, 1, g, V, Jl, &options, st, stream);
        }
        if (status == MPF_OK || status == MPF_ENOCONV) {
            dataType* Vd = nullptr;
            detail::cuda(cudaMallocAsync((void**)&Vd, sizeof(dataType) * (size_t)Mm * Md, stream), where);
            detail::convert_device(Vd, V, (size_t)Mm * Md, stream, where);
            detail::cuda(cudaMemcpy2DAsync(result->deviceData, sizeof(dataType) * result->dataRows, Vd,
                                           sizeof(dataType) * Mm, sizeof(dataType) * Mm, Md, cudaMemcpyDeviceToDevice,
                                           stream),
                         where);
            cudaFreeAsync(Vd, stream);
            detail::convert_device(jacobian->deviceData, Jl, nJ, stream, where);
            fieldsValid_ = true;
        }
        cudaFreeAsync(V, stream);
        cudaFreeAsync(g, stream);
        cudaFreeAsync(Jl, stream);
        return status;
    }

    mpf_eit_t model_ = nullptr;
    mpf_eit_info info_{};
    bool fieldsValid_ = false;
};

}  // namespace models

namespace solver {

// Regularised inverse step (src/solver/inverse.cpp); the system is solved
// exactly by mpf_inverse_solve (dual form for R = I).
template <class dataType, template <class> class numericalSolverType = numeric::ConjugateGradient>
class Inverse {
public:
    enum RegularizationType { identity, noser, laplacian };

    Inverse(std::shared_ptr<numeric::IrregularMesh const> const mesh,
            std::shared_ptr<numeric::Matrix<dataType> const> const jacobian, dataType const referenceValue,
            unsigned const parallelImages, cublasHandle_t const handle, cudaStream_t const stream)
        : referenceValue(referenceValue), mesh(mesh), parallelImages_(parallelImages) {
        if (!mesh) throw std::invalid_argument("mpFlow::solver::Inverse::Inverse: mesh == nullptr");
        if (parallelImages == 0) throw std::invalid_argument("mpFlow::solver::Inverse::Inverse: parallelImages == 0");
        result = std::make_shared<numeric::Matrix<dataType>>(mesh->elements.rows(), parallelImages, stream);
        updateJacobian(jacobian, handle, stream);
    }

    void updateJacobian(std::shared_ptr<numeric::Matrix<dataType> const> const jacobian, cublasHandle_t const,
                        cudaStream_t const) {
        if (!jacobian) throw std::invalid_argument("mpFlow::solver::Inverse::updateJacobian: jacobian == nullptr");
        if (!jacobian->owner)
            throw std::invalid_argument("mpFlow::solver::Inverse::updateJacobian: jacobian does not come from a model");
        this->jacobian = jacobian;
    }

    std::shared_ptr<numeric::Matrix<dataType> const> solve(
        std::vector<std::shared_ptr<numeric::Matrix<dataType>>> const& calculation,
        std::vector<std::shared_ptr<numeric::Matrix<dataType>>> const& measurement, cublasHandle_t const,
        cudaStream_t const stream, unsigned const maxIterations = 0, unsigned* const iterations = nullptr) {
        (void)maxIterations;
        if (calculation.size() != parallelImages_ || measurement.size() != parallelImages_)
            throw std::invalid_argument("mpFlow::solver::Inverse::solve: wrong number of images");
        const unsigned Mm = calculation[0]->rows, Md = calculation[0]->cols, P = parallelImages_;
        const size_t per = (size_t)Mm * Md, w = sizeof(dataType);
        dataType *calc = nullptr, *meas = nullptr, *out = nullptr;
        detail::cuda(cudaMallocAsync((void**)&calc, w * per * P * 2, stream), "mpFlow::solver::Inverse::solve");
        meas = calc + per * P;
        const unsigned E = mesh->elements.rows();
        detail::cuda(cudaMallocAsync((void**)&out, w * (size_t)E * P, stream), "mpFlow::solver::Inverse::solve");
        for (unsigned p = 0; p < P; ++p) {
            cudaMemcpy2DAsync(calc + p * per, w * Mm, calculation[p]->deviceData, w * calculation[p]->dataRows, w * Mm,
                              Md, cudaMemcpyDeviceToDevice, stream);
            cudaMemcpy2DAsync(meas + p * per, w * Mm, measurement[p]->deviceData, w * measurement[p]->dataRows, w * Mm,
                              Md, cudaMemcpyDeviceToDevice, stream);
        }
        const double factor = detail::real_part(regularizationFactor_);
        int st;
        if constexpr (detail::lib_native<dataType>()) {
            // float, thrust::complex<float>, std::complex<float>: the library's own precision
            if constexpr (detail::is_complex<dataType>::value)
                st = mpf_inverse_solve_complex(jacobian->owner, (int32_t)regularizationType_, factor, (int32_t)P,
                                               reinterpret_cast<const float*>(jacobian->deviceData),
                                               reinterpret_cast<const float*>(calc),
                                               reinterpret_cast<const float*>(meas), reinterpret_cast<float*>(out),
                                               stream);
            else
                st = mpf_inverse_solve(jacobian->owner, (int32_t)regularizationType_, factor, (int32_t)P,
                                       jacobian->deviceData, calc, meas, out, stream);
        } else {
            st = solve_converted(factor, calc, per * P, E, out, stream);
        }
        if (st == MPF_OK)
            cudaMemcpy2DAsync(result->deviceData, w * result->dataRows, out, w * E, w * E, P, cudaMemcpyDeviceToDevice,
                              stream);
        cudaFreeAsync(calc, stream);
        cudaFreeAsync(out, stream);
        detail::check(st, "mpFlow::solver::Inverse::solve");
        detail::cuda(cudaStreamSynchronize(stream), "mpFlow::solver::Inverse::solve");
        if (iterations) *iterations = 1;  // one exact solve
        return result;
    }

    void setRegularizationFactor(dataType const factor, cublasHandle_t const, cudaStream_t const) {
        regularizationFactor_ = factor;
    }
    void setRegularizationType(RegularizationType const type, cublasHandle_t const, cudaStream_t const) {
        regularizationType_ = type;
    }
    void setRegularizationParameter(dataType const factor, RegularizationType const type, cublasHandle_t const,
                                    cudaStream_t const) {
        regularizationFactor_ = factor;
        regularizationType_ = type;
    }
    dataType regularizationFactor() const { return regularizationFactor_; }
    RegularizationType regularizationType() const { return regularizationType_; }

    dataType const referenceValue;

private:
    // double, complex<double>: through the library's FP32 interface; calc
    // holds the calculation images followed by the measurement images
    // (`images` values each), out receives E x P results
    int solve_converted(double factor, dataType const* calc, size_t images, unsigned E, dataType* out,
                        cudaStream_t const stream) {
        typedef detail::lib_type<dataType> L;
        const char* where = "mpFlow::solver::Inverse::solve";
        const size_t nJ = (size_t)jacobian->dataRows * E, nOut = (size_t)E * parallelImages_;
        L *calcL = nullptr, *JL = nullptr, *outL = nullptr;
        detail::cuda(cudaMallocAsync((void**)&calcL, sizeof(L) * images * 2, stream), where);
        detail::cuda(cudaMallocAsync((void**)&JL, sizeof(L) * nJ, stream), where);
        detail::cuda(cudaMallocAsync((void**)&outL, sizeof(L) * nOut, stream), where);
        detail::convert_device(calcL, calc, images * 2, stream, where);
        detail::convert_device(JL, jacobian->deviceData, nJ, stream, where);
        int st;
        if constexpr (detail::is_complex<dataType>::value)
            st = mpf_inverse_solve_complex(jacobian->owner, (int32_t)regularizationType_, factor,
                                           (int32_t)parallelImages_, reinterpret_cast<const float*>(JL),
                                           reinterpret_cast<const float*>(calcL),
                                           reinterpret_cast<const float*>(calcL + images),
                                           reinterpret_cast<float*>(outL), stream);
        else
            st = mpf_inverse_solve(jacobian->owner, (int32_t)regularizationType_, factor, (int32_t)parallelImages_,
                                   JL, calcL, calcL + images, outL, stream);
        if (st == MPF_OK) detail::convert_device(out, outL, nOut, stream, where);
        cudaFreeAsync(calcL, stream);
        cudaFreeAsync(JL, stream);
        cudaFreeAsync(outL, stream);
        return st;
    }

    std::shared_ptr<numeric::IrregularMesh const> const mesh;
    std::shared_ptr<numeric::Matrix<dataType> const> jacobian;
    std::shared_ptr<numeric::Matrix<dataType>> result;
    unsigned const parallelImages_;
    dataType regularizationFactor_ = dataType(0);
    RegularizationType regularizationType_ = identity;
};

// Difference and absolute reconstruction (src/solver/solver.cpp).
template <class forwardModelType = models::EIT<>,
          template <class> class numericalInverseSolverType = numeric::ConjugateGradient>
class Solver {
public:
    typedef typename forwardModelType::dataType dataType;

    Solver(std::shared_ptr<forwardModelType> const forwardModel, unsigned const parallelImages,
           cublasHandle_t const handle, cudaStream_t const stream)
        : forwardModel(forwardModel) {
        if (!forwardModel) throw std::invalid_argument("mpFlow::solver::Solver::Solver: forwardModel == nullptr");
        if (parallelImages == 0) throw std::invalid_argument("mpFlow::solver::Solver::Solver: parallelImages == 0");
        const unsigned Mm = forwardModel->result->rows, Md = forwardModel->result->cols;
        for (unsigned p = 0; p < parallelImages; ++p) {
            measurement.push_back(std::make_shared<numeric::Matrix<dataType>>(Mm, Md, stream));
            calculation.push_back(std::make_shared<numeric::Matrix<dataType>>(Mm, Md, stream));
        }
        const unsigned E = forwardModel->mesh->elements.rows();
        const dataType start = forwardModelType::logarithmic ? dataType(0) : dataType(1);
        referenceDistribution = std::make_shared<numeric::Matrix<dataType>>(E, 1, stream, start);
        materialDistribution = std::make_shared<numeric::Matrix<dataType>>(E, 1, stream, start);
        inverseSolver = std::make_shared<Inverse<dataType, numericalInverseSolverType>>(
            forwardModel->mesh, forwardModel->jacobian, forwardModel->referenceValue, parallelImages, handle, stream);
    }

    // src/solver/solver.cpp:64-135: {"model": ..., "solver": {"parallelImages",
    // "regularizationFactor", "regularizationType"}}; the model's "material"
    // may name a reference distribution file and "noSensitivity" a 0/1 mask
    // of the Jacobian.  Ends with preSolve.
    static std::shared_ptr<Solver<forwardModelType, numericalInverseSolverType>> fromConfig(
        json::value const& config, cublasHandle_t const handle, cudaStream_t const stream, std::string const path = "./",
        std::shared_ptr<numeric::IrregularMesh const> const externalMesh = nullptr) {
        auto const& modelConfig = config["model"];
        auto const& solverConfig = config["solver"];
        auto const forwardModel = forwardModelType::fromConfig(modelConfig, handle, stream, path, externalMesh);
        std::shared_ptr<numeric::Matrix<dataType>> reference;
        if (modelConfig["material"].type == json::value::string)
            reference = numeric::Matrix<dataType>::loadtxt(path + "/" + modelConfig["material"].str, stream);
        else if (modelConfig["material"]["distribution"].type == json::value::string)
            reference = numeric::Matrix<dataType>::loadtxt(path + "/" + modelConfig["material"]["distribution"].str, stream);
        const unsigned parallelImages = (unsigned)std::max(1L, solverConfig["parallelImages"].asInt(1));
        auto solver = std::make_shared<Solver<forwardModelType, numericalInverseSolverType>>(forwardModel, parallelImages,
                                                                                            handle, stream);
        if (reference) solver->referenceDistribution = reference;
        solver->preSolve(handle, stream);
        if (modelConfig["noSensitivity"].type == json::value::string) {
            auto mask = numeric::Matrix<dataType>::loadtxt(path + "/" + modelConfig["noSensitivity"].str, stream);
            forwardModel->maskJacobian(mask, stream);
            solver->inverseSolver->updateJacobian(forwardModel->jacobian, handle, stream);
        }
        const std::string type = solverConfig["regularizationType"].asString();
        typedef Inverse<dataType, numericalInverseSolverType> inverseType;
        solver->inverseSolver->setRegularizationParameter(
            (dataType)solverConfig["regularizationFactor"].asDouble(),
            type == "noser" ? inverseType::noser : type == "laplacian" ? inverseType::laplacian : inverseType::identity,
            handle, stream);
        return solver;
    }

    // forward solve at the reference distribution; measurement and
    // calculation start from its voltages (src/solver/solver.cpp:142-166)
    void preSolve(cublasHandle_t const handle, cudaStream_t const stream) {
        auto const initial = forwardModel->solve(referenceDistribution, handle, stream);
        inverseSolver->updateJacobian(forwardModel->jacobian, handle, stream);
        for (auto& m : measurement) m->copy(initial, stream);
        for (auto& c : calculation) c->copy(initial, stream);
        detail::cuda(cudaStreamSynchronize(stream), "mpFlow::solver::Solver::preSolve");
    }

    std::shared_ptr<numeric::Matrix<dataType> const> solveDifferential(cublasHandle_t const handle,
                                                                        cudaStream_t const stream,
                                                                        unsigned const maxIterations = 0,
                                                                        unsigned* const iterations = nullptr) {
        auto const result = inverseSolver->solve(calculation, measurement, handle, stream, maxIterations, iterations);
        add_first_column(result, referenceDistribution, stream);
        return materialDistribution;
    }

    std::shared_ptr<numeric::Matrix<dataType> const> solveAbsolute(cublasHandle_t const handle,
                                                                    cudaStream_t const stream,
                                                                    unsigned const maxIterations = 0,
                                                                    unsigned* const iterations = nullptr) {
        if (measurement.size() != 1)
            throw std::runtime_error("mpFlow::solver::Solver::solveAbsolute: parallelImages != 1");
        forwardModel->solve(materialDistribution, handle, stream);
        inverseSolver->updateJacobian(forwardModel->jacobian, handle, stream);
        calculation[0]->copy(forwardModel->result, stream);
        auto const result = inverseSolver->solve(calculation, measurement, handle, stream, maxIterations, iterations);
        add_first_column(result, materialDistribution, stream);
        return materialDistribution;
    }

    std::shared_ptr<forwardModelType> const forwardModel;
    std::shared_ptr<Inverse<dataType, numericalInverseSolverType>> inverseSolver;
    std::vector<std::shared_ptr<numeric::Matrix<dataType>>> measurement;
    std::vector<std::shared_ptr<numeric::Matrix<dataType>>> calculation;
    std::shared_ptr<numeric::Matrix<dataType>> referenceDistribution;
    std::shared_ptr<numeric::Matrix<dataType>> materialDistribution;

private:
    // materialDistribution = base + first column of delta (host round trip: E values)
    void add_first_column(std::shared_ptr<numeric::Matrix<dataType> const> const delta,
                          std::shared_ptr<numeric::Matrix<dataType> const> const base, cudaStream_t const stream) {
        const unsigned E = base->rows;
        std::vector<dataType> a(E), b(E);
        cudaMemcpyAsync(a.data(), base->deviceData, sizeof(dataType) * E, cudaMemcpyDeviceToHost, stream);
        cudaMemcpyAsync(b.data(), delta->deviceData, sizeof(dataType) * E, cudaMemcpyDeviceToHost, stream);
        detail::cuda(cudaStreamSynchronize(stream), "mpFlow::solver::Solver");
        for (unsigned i = 0; i < E; ++i) a[i] += b[i];
        detail::cuda(cudaMemcpyAsync(materialDistribution->deviceData, a.data(), sizeof(dataType) * E,
                                     cudaMemcpyHostToDevice, stream),
                     "mpFlow::solver::Solver");
        detail::cuda(cudaStreamSynchronize(stream), "mpFlow::solver::Solver");
    }
};

}  // namespace solver
}  // namespace mpFlow
