// extern "C" entry points of libmpflow_gb300 (declared in include/mpflow_gb300.h).
// Every entry catches C++ exceptions so none crosses the ABI, and records a
// thread-local message for mpf_last_error().
#include <cuda_runtime.h>

#include <atomic>
#include <exception>
#include <new>

#include "model.h"

namespace mpf {

static thread_local std::string g_error;
static std::atomic<long long> g_launches{0};

void add_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launches() { return g_launches.load(std::memory_order_relaxed); }

void set_error(const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_error = buf;
}

int fail(int status, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_error = buf;
    return status;
}

const char* last_error() { return g_error.c_str(); }

int eit_create(const mpf_eit_desc* d, mpf_eit** out);
int eit_assemble_export(mpf_eit* m, int F, const float* gamma, float* sOut, float* rOut, cudaStream_t s);
int eit_forward(mpf_eit* m, int F, const float* gamma, float* V, float* Jref, const mpf_solve_opts* o,
                mpf_solve_stats* stats, cudaStream_t s);
int eit_fields(mpf_eit* m, int F, float* out, cudaStream_t s);
int eit_fields_complex(mpf_eit* m, int F, float* out, cudaStream_t s);
int eit_forward_complex(mpf_eit* m, int F, const float* gamma, float* Vout, float* Jref, const mpf_solve_opts* optsIn,
                        mpf_solve_stats* stats, cudaStream_t s);
int gn_step(mpf_eit* m, int F, float* gamma, const float* vMeas, double lambda, const mpf_solve_opts* o,
            double* residual, mpf_solve_stats* stats, cudaStream_t s);
void eit_info(const mpf_eit* m, mpf_eit_info* i);
void eit_destroy(mpf_eit* m);
int gn_solve(mpf_eit* m, int F, float* gamma, const float* vMeas, double lambda, double target, int maxIters,
             const mpf_solve_opts* o, int32_t* itersOut, double* resOut, mpf_gn_stats* stats, cudaStream_t s);
int profile_cg(mpf_eit* m, int F, const float* gamma, int reps, double* ms, double* bytes, cudaStream_t s);
int profile_cg_loop(mpf_eit* m, int F, const float* gamma, int graphs, double* ms, cudaStream_t s);
int phase_times(mpf_eit* m, int enable, double* ms, int cap, int64_t* calls);
int profile_fem(mpf_eit* m, int F, const float* gamma, int reps, double* ms, double* bytes, cudaStream_t s);
int group_iterations(mpf_eit* m, int32_t* out, int cap, int32_t* count);
int cg_variants(mpf_eit* m, const int32_t* set, int F, int32_t* get);
int wait_selftest(int timeoutUs, cudaStream_t s);
int batch_create(mpf_eit* const* models, int count, mpf_batch** out);
int matrix_elementwise(int op, int rows, int cols, const float* A, const float* B, float* C, int ld, float scalar,
                       cudaStream_t s);
int matrix_column_reduce(int op, int rows, int cols, const float* A, const float* B, int ld, float* result, int ldr,
                         cudaStream_t s);
int matrix_multiply(int transA, int transB, int m, int n, int k, const float* A, int lda, const float* B, int ldb,
                    float* C, int ldc, cudaStream_t s);
int sparse_create(int rows, const float* values, const uint32_t* columnIds, uint32_t density, mpf_sparse** out);
void sparse_destroy(mpf_sparse* A);
int sparse_multiply(mpf_sparse* A, const float* x, int ldx, int cols, float* y, int ldy, cudaStream_t s);
int sparse_solve(mpf_sparse* A, int solver, const float* b, int ldb, float* x, int ldx, int cols, int maxIter,
                 double tol, int dcFree, int32_t* iterations, cudaStream_t s);
int batch_forward(mpf_batch* b, int F, const float* const* gamma, float* const* V, const mpf_solve_opts* in,
                  mpf_solve_stats* stats, cudaStream_t s);
int batch_iterations(mpf_batch* b, int32_t* out, int cap, int32_t* count);
int batch_cg_stats(mpf_batch* b, double* ms, double* bytes);
int batch_cg_variants(mpf_batch* b, const int32_t* set, int F, int32_t* get, int cap, int32_t* classes);
void batch_destroy(mpf_batch* b);
int inverse_solve(mpf_eit* m, int reg, double factor, int images, const float* Jref, const float* calc,
                  const float* meas, float* result, cudaStream_t s);
int mlp_create(int in, int h1, int h2, int out, unsigned long long seed, int device, mpf_mlp** res);
void mlp_destroy(mpf_mlp* n);
void mlp_layout(const mpf_mlp* n, int64_t* off);
int mlp_forward(mpf_mlp* n, int batch, const float* x, float* y, int ldy, cudaStream_t s);
int mlp_backward(mpf_mlp* n, int batch, const float* x, const float* target, int ldt, int tvalid, double* loss,
                 cudaStream_t s);
int mlp_adam(mpf_mlp* n, float lr, float beta1, float beta2, float eps, float weightDecay, cudaStream_t s);
int mlp_train_step(mpf_mlp* n, int batch, const float* x, int ldx, const int* rows, const float* target, int ldt,
                   int tvalid, float lr, float beta1, float beta2, float eps, float weightDecay, double* loss,
                   cudaStream_t s);
int mlp_params(mpf_mlp* n, float* buf, int which, cudaStream_t s);
int learned_input(mpf_eit* m, int F, const float* vMeas, float* x, cudaStream_t s);
int learned_prior(mpf_eit* m, double lambda, cudaStream_t s);
int inverse_solve_complex(mpf_eit* m, int reg, double factor, int images, const float* Jref, const float* calc,
                          const float* meas, float* result, cudaStream_t s);
int learned_prior_apply(mpf_eit* m, int F, const float* x, float* out, int ldo, int mode, cudaStream_t s);
int gn_solve_learned(mpf_eit* m, mpf_mlp* net, int F, float* gamma, const float* vMeas, double lambda,
                     double target, int maxIters, const mpf_solve_opts* o, int32_t* itersOut, double* resOut,
                     int32_t* accepted, mpf_gn_stats* stats, cudaStream_t s);

}  // namespace mpf

#define MPF_GUARD(...)                                                         \
    try {                                                                      \
        mpf::set_error("%s", "");                                              \
        __VA_ARGS__                                                            \
    } catch (const std::bad_alloc&) {                                          \
        return mpf::fail(MPF_ENOMEM, "host allocation failed");                \
    } catch (const std::exception& ex) {                                       \
        return mpf::fail(MPF_EINVAL, "%s", ex.what());                         \
    } catch (...) {                                                            \
        return mpf::fail(MPF_EINVAL, "unknown C++ exception");                 \
    }

extern "C" {

const char* mpf_last_error(void) { return mpf::last_error(); }

const char* mpf_version(void) { return "mpflow_gb300 0.1.0 (sm_103a)"; }

long long mpf_kernel_launches(void) { return mpf::launches(); }

int mpf_selftest_bounded_wait(int32_t timeout_us, mpf_stream_t stream) {
    MPF_GUARD({ return mpf::wait_selftest(timeout_us, (cudaStream_t)stream); })
}

uint32_t mpf_data_rows(uint32_t rows) { return mpf::data_rows(rows); }

int mpf_ring_mesh_counts(int32_t rings, int32_t* n_nodes, int32_t* n_elements) {
    MPF_GUARD({
        MPF_CHECK(rings >= 1 && rings <= 2000 && n_nodes && n_elements, MPF_EINVAL,
                  "mpf_ring_mesh_counts: rings must be in [1, 2000]");
        *n_nodes = 1 + 3 * rings * (rings + 1);
        *n_elements = 6 * rings * rings;
        return MPF_OK;
    })
}

int mpf_ring_mesh(int32_t rings, double radius, double* nodes, int32_t* elements) {
    MPF_GUARD({
        MPF_CHECK(nodes && elements, MPF_EINVAL, "mpf_ring_mesh: null output");
        return mpf::ring_mesh(rings, radius, nodes, elements);
    })
}

int mpf_mesh_edges(int32_t n_nodes, int32_t n_elements, const double* nodes, const int32_t* elements,
                   int32_t* edges, int32_t* element_edges, int32_t* boundary, int32_t* n_edges,
                   int32_t* n_boundary) {
    MPF_GUARD({
        MPF_CHECK(nodes && elements && edges && element_edges && boundary && n_edges && n_boundary, MPF_EINVAL,
                  "mpf_mesh_edges: null argument");
        return mpf::mesh_edges(n_nodes, n_elements, nodes, elements, edges, element_edges, boundary, n_edges,
                               n_boundary);
    })
}

int mpf_ports_circular(int32_t n_nodes, const double* nodes, int32_t n_elements, const int32_t* elements,
                       const int32_t* edges, int32_t n_boundary, const int32_t* boundary, int32_t count, double width,
                       double offset, int32_t clockwise, int32_t* port_edges, int32_t cap, int32_t* max_port_edges) {
    MPF_GUARD({
        MPF_CHECK(nodes && elements && edges && boundary && port_edges && max_port_edges, MPF_EINVAL,
                  "mpf_ports_circular: null argument");
        return mpf::ports_circular(n_nodes, nodes, n_elements, elements, edges, n_boundary, boundary, count, width,
                                   offset, clockwise, port_edges, cap, max_port_edges);
    })
}

int mpf_p1_elemental(int32_t n_elements, const double* nodes, const int32_t* elements, double* stiffness,
                     double* mass) {
    MPF_GUARD({
        MPF_CHECK(n_elements > 0 && nodes && elements && stiffness && mass, MPF_EINVAL,
                  "mpf_p1_elemental: bad arguments");
        mpf::p1_elemental(n_elements, nodes, elements, stiffness, mass);
        return MPF_OK;
    })
}

int mpf_ell_layout(int32_t n_nodes, int32_t n_elements, const int32_t* elements, uint32_t* column_ids,
                   uint32_t* density) {
    MPF_GUARD({
        MPF_CHECK(elements && column_ids && density, MPF_EINVAL, "mpf_ell_layout: null argument");
        mpf::FemStructure fs;
        MPF_TRY(mpf::build_structure(n_nodes, n_elements, elements, fs));
        std::copy(fs.refColIds.begin(), fs.refColIds.end(), column_ids);
        *density = (uint32_t)fs.density;
        return MPF_OK;
    })
}

int mpf_excitation_matrix(int32_t n_nodes, const double* nodes, const int32_t* edges, int32_t ports,
                          const int32_t* port_edges, int32_t cap, double* exc, int32_t ld) {
    MPF_GUARD({
        MPF_CHECK(nodes && edges && port_edges && exc && ld >= n_nodes && ports > 0, MPF_EINVAL,
                  "mpf_excitation_matrix: bad arguments");
        mpf::excitation_matrix(n_nodes, nodes, edges, ports, port_edges, cap, exc, ld);
        return MPF_OK;
    })
}

int mpf_eit_create(const mpf_eit_desc* desc, mpf_eit_t* model) {
    MPF_GUARD({
        MPF_CHECK(model, MPF_EINVAL, "mpf_eit_create: model == nullptr");
        *model = nullptr;
        return mpf::eit_create(desc, model);
    })
}

int mpf_eit_destroy(mpf_eit_t model) {
    MPF_GUARD({
        mpf::eit_destroy(model);
        return MPF_OK;
    })
}

int mpf_eit_get_info(mpf_eit_t model, mpf_eit_info* info) {
    MPF_GUARD({
        MPF_CHECK(model && info, MPF_EINVAL, "mpf_eit_get_info: null argument");
        mpf::eit_info(model, info);
        return MPF_OK;
    })
}

int mpf_eit_assemble(mpf_eit_t model, int32_t frames, const float* gamma, float* s_values, float* r_values,
                     mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(model, MPF_EINVAL, "mpf_eit_assemble: model == nullptr");
        return mpf::eit_assemble_export(model, frames, gamma, s_values, r_values, (cudaStream_t)stream);
    })
}

int mpf_eit_forward(mpf_eit_t model, int32_t frames, const float* gamma, float* voltages, float* jacobian,
                    const mpf_solve_opts* opts, mpf_solve_stats* stats, mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(model, MPF_EINVAL, "mpf_eit_forward: model == nullptr");
        return mpf::eit_forward(model, frames, gamma, voltages, jacobian, opts, stats, (cudaStream_t)stream);
    })
}

int mpf_eit_forward_complex(mpf_eit_t model, int32_t frames, const float* gamma, float* voltages, float* jacobian,
                            const mpf_solve_opts* opts, mpf_solve_stats* stats, mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(model, MPF_EINVAL, "mpf_eit_forward_complex: model == nullptr");
        return mpf::eit_forward_complex(model, frames, gamma, voltages, jacobian, opts, stats, (cudaStream_t)stream);
    })
}

int mpf_eit_fields(mpf_eit_t model, int32_t frames, float* fields, mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(model, MPF_EINVAL, "mpf_eit_fields: model == nullptr");
        return mpf::eit_fields(model, frames, fields, (cudaStream_t)stream);
    })
}

int mpf_eit_fields_complex(mpf_eit_t model, int32_t frames, float* fields, mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(model, MPF_EINVAL, "mpf_eit_fields_complex: model == nullptr");
        return mpf::eit_fields_complex(model, frames, fields, (cudaStream_t)stream);
    })
}

int mpf_gn_step(mpf_eit_t model, int32_t frames, float* gamma, const float* v_meas, double lambda,
                const mpf_solve_opts* opts, double* residual, mpf_solve_stats* stats, mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(model, MPF_EINVAL, "mpf_gn_step: model == nullptr");
        MPF_CHECK(lambda >= 0.0, MPF_EINVAL, "mpf_gn_step: lambda < 0");
        return mpf::gn_step(model, frames, gamma, v_meas, lambda, opts, residual, stats, (cudaStream_t)stream);
    })
}

int mpf_gn_solve(mpf_eit_t model, int32_t frames, float* gamma, const float* v_meas, double lambda, double target,
                 int32_t max_gn_iters, const mpf_solve_opts* opts, int32_t* iterations, double* residual,
                 mpf_gn_stats* stats, mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(model, MPF_EINVAL, "mpf_gn_solve: model == nullptr");
        MPF_CHECK(lambda >= 0.0 && target >= 0.0, MPF_EINVAL, "mpf_gn_solve: lambda and target must be >= 0");
        return mpf::gn_solve(model, frames, gamma, v_meas, lambda, target, max_gn_iters, opts, iterations, residual,
                             stats, (cudaStream_t)stream);
    })
}

int mpf_eit_profile_fem(mpf_eit_t model, int32_t frames, const float* gamma, int32_t reps, double* ms,
                        double* bytes, mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(model, MPF_EINVAL, "mpf_eit_profile_fem: model == nullptr");
        return mpf::profile_fem(model, frames, gamma, reps, ms, bytes, (cudaStream_t)stream);
    })
}

int mpf_eit_profile_cg(mpf_eit_t model, int32_t frames, const float* gamma, int32_t reps, double* ms, double* bytes,
                       mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(model, MPF_EINVAL, "mpf_eit_profile_cg: model == nullptr");
        return mpf::profile_cg(model, frames, gamma, reps, ms, bytes, (cudaStream_t)stream);
    })
}

int mpf_eit_profile_cg_loop(mpf_eit_t model, int32_t frames, const float* gamma, int32_t graphs, double* ms,
                            mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(model, MPF_EINVAL, "mpf_eit_profile_cg_loop: model == nullptr");
        return mpf::profile_cg_loop(model, frames, gamma, graphs, ms, (cudaStream_t)stream);
    })
}

int mpf_eit_phase_times(mpf_eit_t model, int32_t enable, double* ms, int32_t cap, int64_t* calls) {
    MPF_GUARD({
        MPF_CHECK(model, MPF_EINVAL, "mpf_eit_phase_times: model == nullptr");
        return mpf::phase_times(model, enable, ms, cap, calls);
    })
}

int mpf_eit_group_iterations(mpf_eit_t model, int32_t* iterations, int32_t cap, int32_t* count) {
    MPF_GUARD({
        MPF_CHECK(model, MPF_EINVAL, "mpf_eit_group_iterations: model == nullptr");
        return mpf::group_iterations(model, iterations, cap, count);
    })
}

int mpf_eit_cg_variants(mpf_eit_t model, const int32_t* set, int32_t frames, int32_t* get) {
    MPF_GUARD({
        MPF_CHECK(model, MPF_EINVAL, "mpf_eit_cg_variants: model == nullptr");
        return mpf::cg_variants(model, set, frames, get);
    })
}

int mpf_matrix_elementwise(int32_t op, int32_t rows, int32_t cols, const float* A, const float* B, float* C,
                           int32_t ld, float scalar, mpf_stream_t stream) {
    MPF_GUARD({ return mpf::matrix_elementwise(op, rows, cols, A, B, C, ld, scalar, (cudaStream_t)stream); })
}

int mpf_convert_values(int32_t direction, int64_t count, const void* src, void* dst, mpf_stream_t stream) {
    MPF_GUARD({ return mpf::convert_values(direction, (long long)count, src, dst, (cudaStream_t)stream); })
}

int mpf_matrix_column_reduce(int32_t op, int32_t rows, int32_t cols, const float* A, const float* B, int32_t ld,
                             float* result, int32_t ldr, mpf_stream_t stream) {
    MPF_GUARD({ return mpf::matrix_column_reduce(op, rows, cols, A, B, ld, result, ldr, (cudaStream_t)stream); })
}

int mpf_matrix_multiply(int32_t trans_a, int32_t trans_b, int32_t m, int32_t n, int32_t k, const float* A,
                        int32_t lda, const float* B, int32_t ldb, float* C, int32_t ldc, mpf_stream_t stream) {
    MPF_GUARD({
        return mpf::matrix_multiply(trans_a, trans_b, m, n, k, A, lda, B, ldb, C, ldc, (cudaStream_t)stream);
    })
}

int mpf_sparse_create(int32_t rows, const float* values, const uint32_t* column_ids, uint32_t density,
                      mpf_sparse_t* matrix) {
    MPF_GUARD({ return mpf::sparse_create(rows, values, column_ids, density, matrix); })
}

int mpf_sparse_destroy(mpf_sparse_t matrix) {
    MPF_GUARD({
        mpf::sparse_destroy(matrix);
        return MPF_OK;
    })
}

int mpf_sparse_multiply(mpf_sparse_t matrix, const float* x, int32_t ldx, int32_t cols, float* y, int32_t ldy,
                        mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(matrix, MPF_EINVAL, "mpFlow::numeric::SparseMatrix::multiply: matrix == nullptr");
        return mpf::sparse_multiply(matrix, x, ldx, cols, y, ldy, (cudaStream_t)stream);
    })
}

int mpf_sparse_solve(mpf_sparse_t matrix, int32_t solver, const float* b, int32_t ldb, float* x, int32_t ldx,
                     int32_t cols, int32_t max_iter, double tol, int32_t dc_free, int32_t* iterations,
                     mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(matrix, MPF_EINVAL, "mpFlow::numeric::ConjugateGradient::solve: A == nullptr");
        return mpf::sparse_solve(matrix, solver, b, ldb, x, ldx, cols, max_iter, tol, dc_free, iterations,
                                 (cudaStream_t)stream);
    })
}

int mpf_batch_create(const mpf_eit_t* models, int32_t count, mpf_batch_t* batch) {
    MPF_GUARD({
        MPF_CHECK(models && batch && count >= 1, MPF_EINVAL, "mpf_batch_create: bad arguments");
        return mpf::batch_create(models, count, batch);
    })
}

int mpf_batch_destroy(mpf_batch_t batch) {
    MPF_GUARD({
        mpf::batch_destroy(batch);
        return MPF_OK;
    })
}

int mpf_batch_forward(mpf_batch_t batch, int32_t frames, const float* const* gamma, float* const* voltages,
                      const mpf_solve_opts* opts, mpf_solve_stats* stats, mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(batch, MPF_EINVAL, "mpf_batch_forward: batch == nullptr");
        return mpf::batch_forward(batch, frames, gamma, voltages, opts, stats, (cudaStream_t)stream);
    })
}

int mpf_batch_iterations(mpf_batch_t batch, int32_t* iterations, int32_t cap, int32_t* count) {
    MPF_GUARD({
        MPF_CHECK(batch && (iterations || cap == 0), MPF_EINVAL, "mpf_batch_iterations: bad arguments");
        return mpf::batch_iterations(batch, iterations, cap, count);
    })
}

int mpf_batch_cg_stats(mpf_batch_t batch, double* cg_ms, double* cg_bytes) {
    MPF_GUARD({
        MPF_CHECK(batch, MPF_EINVAL, "mpf_batch_cg_stats: batch == nullptr");
        return mpf::batch_cg_stats(batch, cg_ms, cg_bytes);
    })
}

int mpf_batch_cg_variants(mpf_batch_t batch, const int32_t* set, int32_t frames, int32_t* get, int32_t cap,
                          int32_t* classes) {
    MPF_GUARD({
        MPF_CHECK(batch && frames >= 1, MPF_EINVAL, "mpf_batch_cg_variants: bad arguments");
        return mpf::batch_cg_variants(batch, set, frames, get, cap, classes);
    })
}

int mpf_gram_split_bf16(int32_t batch, int32_t rows, int32_t cols, const float* A, int32_t lda, float* C,
                        mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(batch >= 1 && A && C && lda >= cols, MPF_EINVAL, "mpf_gram_split_bf16: bad arguments");
        MPF_CHECK(rows % 128 == 0 && cols % 64 == 0 && lda % 8 == 0, MPF_EINVAL,
                  "mpf_gram_split_bf16: rows %% 128, cols %% 64 and lda %% 8 must be 0");
        cudaStream_t s = (cudaStream_t)stream;
        mpf::DevBuf<__nv_bfloat16> hi, lo;
        mpf::DevBuf<float> work;
        MPF_TRY(hi.alloc((size_t)batch * rows * lda));
        MPF_TRY(lo.alloc((size_t)batch * rows * lda));
        MPF_TRY(work.alloc(mpf::dense_gram_work_floats(batch, rows, cols)));
        MPF_TRY(mpf::dense_split_bf16(batch, rows, cols, A, lda, hi.ptr, lo.ptr, s));
        MPF_TRY(mpf::dense_gram_split_bf16(batch, rows, cols, hi.ptr, lo.ptr, lda, C, work.ptr, work.count, s));
        MPF_CUDA(cudaStreamSynchronize(s));
        bool aborted = false;
        MPF_TRY(mpf::dense_gram_check_abort(&aborted));
        MPF_CHECK(!aborted, MPF_ETIMEOUT, "gram kernel: a pipeline wait timed out");
        return MPF_OK;
    })
}

int mpf_profile_gram(int32_t batch, int32_t rows, int32_t cols, int32_t reps, double* ms_per_launch,
                     mpf_stream_t stream) {
    MPF_GUARD({ return mpf::dense_profile_gram(batch, rows, cols, reps, ms_per_launch, (cudaStream_t)stream); })
}

int mpf_gram_split_bf16_noalloc(int32_t batch, int32_t rows, int32_t cols, const float* A, int32_t lda, float* C,
                                mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(A && C, MPF_EINVAL, "mpf_gram_split_bf16_noalloc: null argument");
        return mpf::dense_gram_split_bf16_noalloc(batch, rows, cols, A, lda, C, (cudaStream_t)stream);
    })
}

int mpf_cholesky_solve_f64(int32_t batch, int32_t n, double* A, double shift, double* B, int32_t nrhs,
                           int32_t* info, mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(batch >= 1 && n >= 1 && A && B && info && nrhs >= 1, MPF_EINVAL,
                  "mpf_cholesky_solve_f64: bad arguments");
        cudaStream_t s = (cudaStream_t)stream;
        if (shift != 0.0) MPF_TRY(mpf::dense_add_shift(batch, n, A, shift, s));
        MPF_TRY(mpf::dense_cholesky_f64(batch, n, A, info, s));
        MPF_TRY(mpf::dense_cholesky_solve_f64(batch, n, A, B, nrhs, s));
        return MPF_OK;
    })
}

int mpf_mlp_create(int32_t in, int32_t hidden1, int32_t hidden2, int32_t out, uint64_t seed, int32_t device,
                   mpf_mlp_t* net) {
    MPF_GUARD({ return mpf::mlp_create(in, hidden1, hidden2, out, (unsigned long long)seed, device, net); })
}

int mpf_mlp_destroy(mpf_mlp_t net) {
    MPF_GUARD({
        mpf::mlp_destroy(net);
        return MPF_OK;
    })
}

int mpf_mlp_layout(mpf_mlp_t net, int64_t* offsets) {
    MPF_GUARD({
        MPF_CHECK(net && offsets, MPF_EINVAL, "mpf_mlp_layout: null argument");
        mpf::mlp_layout(net, offsets);
        return MPF_OK;
    })
}

int mpf_mlp_forward(mpf_mlp_t net, int32_t batch, const float* x, float* y, int32_t ldy, mpf_stream_t stream) {
    MPF_GUARD({ return mpf::mlp_forward(net, batch, x, y, ldy, (cudaStream_t)stream); })
}

int mpf_mlp_backward(mpf_mlp_t net, int32_t batch, const float* x, const float* target, int32_t ldt, int32_t valid,
                     double* loss, mpf_stream_t stream) {
    MPF_GUARD({ return mpf::mlp_backward(net, batch, x, target, ldt, valid, loss, (cudaStream_t)stream); })
}

int mpf_mlp_adam(mpf_mlp_t net, float lr, float beta1, float beta2, float eps, float weight_decay,
                 mpf_stream_t stream) {
    MPF_GUARD({ return mpf::mlp_adam(net, lr, beta1, beta2, eps, weight_decay, (cudaStream_t)stream); })
}

int mpf_mlp_train_step(mpf_mlp_t net, int32_t batch, const float* x, int32_t ldx, const int32_t* rows,
                       const float* target, int32_t ldt, int32_t valid, float lr, float beta1, float beta2,
                       float eps, float weight_decay, double* loss, mpf_stream_t stream) {
    MPF_GUARD({
        return mpf::mlp_train_step(net, batch, x, ldx, rows, target, ldt, valid, lr, beta1, beta2, eps, weight_decay,
                                   loss, (cudaStream_t)stream);
    })
}

int mpf_mlp_params(mpf_mlp_t net, float* buffer, int32_t which, mpf_stream_t stream) {
    MPF_GUARD({ return mpf::mlp_params(net, buffer, which, (cudaStream_t)stream); })
}

int mpf_eit_learned_input(mpf_eit_t model, int32_t frames, const float* v_meas, float* x, mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(model, MPF_EINVAL, "mpf_eit_learned_input: model == nullptr");
        return mpf::learned_input(model, frames, v_meas, x, (cudaStream_t)stream);
    })
}

int mpf_inverse_solve_complex(mpf_eit_t model, int32_t regularization, double factor, int32_t images,
                              const float* jacobian, const float* calculation, const float* measurement,
                              float* result, mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(model, MPF_EINVAL, "mpf_inverse_solve_complex: model == nullptr");
        return mpf::inverse_solve_complex(model, regularization, factor, images, jacobian, calculation, measurement,
                                          result, (cudaStream_t)stream);
    })
}

int mpf_eit_learned_prior(mpf_eit_t model, double lambda, mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(model, MPF_EINVAL, "mpf_eit_learned_prior: model == nullptr");
        return mpf::learned_prior(model, lambda, (cudaStream_t)stream);
    })
}

int mpf_eit_learned_prior_apply(mpf_eit_t model, int32_t frames, const float* x, float* out, int32_t ldo,
                                int32_t mode, mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(model, MPF_EINVAL, "mpf_eit_learned_prior_apply: model == nullptr");
        return mpf::learned_prior_apply(model, frames, x, out, ldo, mode, (cudaStream_t)stream);
    })
}

int mpf_gn_solve_learned(mpf_eit_t model, mpf_mlp_t net, int32_t frames, float* gamma, const float* v_meas,
                         double lambda, double target, int32_t max_gn_iters, const mpf_solve_opts* opts,
                         int32_t* iterations, double* residual, int32_t* accepted, mpf_gn_stats* stats,
                         mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(model && net, MPF_EINVAL, "mpf_gn_solve_learned: null model or network");
        MPF_CHECK(lambda >= 0.0 && target >= 0.0, MPF_EINVAL, "mpf_gn_solve_learned: lambda and target must be >= 0");
        return mpf::gn_solve_learned(model, net, frames, gamma, v_meas, lambda, target, max_gn_iters, opts,
                                     iterations, residual, accepted, stats, (cudaStream_t)stream);
    })
}

int mpf_inverse_solve(mpf_eit_t model, int32_t regularization, double factor, int32_t images, const float* jacobian,
                      const float* calculation, const float* measurement, float* result, mpf_stream_t stream) {
    MPF_GUARD({
        MPF_CHECK(model, MPF_EINVAL, "mpFlow::solver::Inverse::solve: model == nullptr");
        return mpf::inverse_solve(model, regularization, factor, images, jacobian, calculation, measurement, result,
                                  (cudaStream_t)stream);
    })
}

}  // extern "C"
