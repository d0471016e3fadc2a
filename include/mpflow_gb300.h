/*
 * mpflow_gb300.h -- C ABI of the GB300-native EIT hot path.
 *
 * One shared library, libmpflow_gb300.so, built for sm_103a.  Every entry
 * point returns an int status (MPF_OK on success); no C++ exception crosses
 * this boundary.  mpf_last_error() gives the message of the last failure on
 * the calling thread.  Device pointers are plain CUDA device addresses owned
 * by the caller; the library owns only the opaque model objects and their
 * workspaces.  All device work is ordered on the stream passed in (a
 * cudaStream_t; NULL is the legacy default stream) and no entry point
 * synchronises the host unless its comment says so.
 *
 * Each declaration names the reference (pgebhardt/mpflow) interface it
 * replaces, as path:line within that project.
 */
#ifndef MPFLOW_GB300_H
#define MPFLOW_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* mpf_stream_t; /* == cudaStream_t */

enum mpf_status {
    MPF_OK = 0,
    MPF_EINVAL = 1,      /* bad argument: the reference throws std::invalid_argument */
    MPF_ENOMEM = 2,      /* device or host allocation failed (std::runtime_error) */
    MPF_ECUDA = 3,       /* a CUDA call failed */
    MPF_ENOCONV = 4,     /* an iterative solve hit its iteration cap */
    MPF_EBREAKDOWN = 5,  /* non-positive pivot / curvature (Cholesky info > 0) */
    MPF_ETIMEOUT = 6,    /* a bounded device-side wait ran out */
    MPF_EFULL = 7,       /* ELL row has more than 32 entries (std::logic_error) */
    MPF_ENOTSUP = 8      /* valid request this library does not implement */
};

/* Source types, include/mpflow/fem/sources.h:31-34 (Sources::Type).  OPEN:
 * current sources, voltages measured.  FIXED: voltage sources, the port
 * nodes carry Dirichlet rows (EIT::applyMixedBoundaryCondition,
 * src/models/eit.cpp:251-270) and the port currents are measured; solved in
 * the equivalent symmetric form (Dirichlet columns eliminated), without FP64
 * refinement and with the reference Jacobian only. */
enum mpf_source_type { MPF_SOURCE_OPEN = 0, MPF_SOURCE_FIXED = 1 };

/* Message of the last failed call on this thread ("" if none). */
const char* mpf_last_error(void);
/* Library version string (src/version.cpp:23-25 analogue). */
const char* mpf_version(void);
/* Number of CUDA kernels this library has launched in the process so far
 * (kernels inside replayed CUDA graphs included).  No reference counterpart
 * (measurement support). */
long long mpf_kernel_launches(void);
/* Failure-path self-test of the bounded device waits (no reference
 * counterpart): a kernel waits on an mbarrier that nothing arrives on, with
 * the wait routine of the tensor-core kernels limited to timeout_us
 * (1..2000000); it gives up, raises its abort flag and returns, so the call
 * returns MPF_ETIMEOUT and the context stays usable.  Synchronises. */
int mpf_selftest_bounded_wait(int32_t timeout_us, mpf_stream_t stream);

/* ======================================================================== */
/* Host-side mesh and FEM setup (no GPU needed)                             */
/* ======================================================================== */

/* Padded row count of a dense matrix: src/numeric/matrix.cpp:49-55 with
 * math::roundTo, include/mpflow/mathematics.h:42-44. */
uint32_t mpf_data_rows(uint32_t rows);

/* Concentric-ring disk mesh: ring i (1..rings) carries 6i nodes, so
 * nodes = 1 + 3 rings (rings+1), elements = 6 rings^2.  Replaces the
 * distmesh branch of IrregularMesh::fromConfig
 * (src/numeric/irregular_mesh.cpp:87-122), whose library is not available.
 * nodes: n x 2 row-major; elements: e x 3 row-major, counter-clockwise. */
int mpf_ring_mesh_counts(int32_t rings, int32_t* n_nodes, int32_t* n_elements);
int mpf_ring_mesh(int32_t rings, double radius, double* nodes, int32_t* elements);

/* Edge table, element->edge map and boundary edge list.  Replaces
 * distmesh::utils::findUniqueEdges / getTriangulationEdgeIndices /
 * fixBoundaryEdgeOrientation / boundEdges used at
 * src/numeric/irregular_mesh.cpp:25-46.  Numbering: elements in order, local
 * edges (0,1),(1,2),(2,0); interior edges stored (min,max); boundary edges
 * oriented counter-clockwise around the domain.  edges: cap 3e x 2,
 * element_edges: e x 3, boundary: cap 3e. */
int mpf_mesh_edges(int32_t n_nodes, int32_t n_elements, const double* nodes,
                   const int32_t* elements, int32_t* edges, int32_t* element_edges,
                   int32_t* boundary, int32_t* n_edges, int32_t* n_boundary);

/* Electrode (port) edge sets on a circular boundary: FEM::Ports::circularBoundary,
 * src/fem/ports.cpp:32-77.  port_edges: count x cap row-major, -1 padded;
 * *max_port_edges receives the widest port. */
int mpf_ports_circular(int32_t n_nodes, const double* nodes, int32_t n_elements,
                       const int32_t* elements, const int32_t* edges, int32_t n_boundary,
                       const int32_t* boundary, int32_t count, double width, double offset,
                       int32_t clockwise, int32_t* port_edges, int32_t cap,
                       int32_t* max_port_edges);

/* P1 elemental stiffness int grad phi_i . grad phi_j and mass int phi_i phi_j,
 * e x 3 x 3 row-major each: basis::Linear::integralA / integralB,
 * src/fem/basis_linear.cpp:72-91. */
int mpf_p1_elemental(int32_t n_elements, const double* nodes, const int32_t* elements,
                     double* stiffness, double* mass);

/* Reference ELL layout of the FEM system matrix: column ids (dataRows x 32,
 * row-major, 0xFFFFFFFF padding) and density, exactly as
 * Equation::initElementalMatrices leaves sMatrix/rMatrix/systemMatrix
 * (src/fem/equation.cpp:131-144, src/numeric/sparse_matrix.cpp:396-423). */
int mpf_ell_layout(int32_t n_nodes, int32_t n_elements, const int32_t* elements,
                   uint32_t* column_ids, uint32_t* density);

/* Excitation matrix (n x ports, column-major, leading dimension ld):
 * Equation::initExcitationMatrix, src/fem/equation.cpp:183-215. */
int mpf_excitation_matrix(int32_t n_nodes, const double* nodes, const int32_t* edges,
                          int32_t ports, const int32_t* port_edges, int32_t cap, double* exc,
                          int32_t ld);

/* ======================================================================== */
/* EIT model: mesh + ports + sources + 2.5D setup, resident on one GPU       */
/* ======================================================================== */

typedef struct mpf_eit* mpf_eit_t;

/* Constructor arguments of models::EIT (include/mpflow/models/eit.h:38-42,
 * src/models/eit.cpp:29-95) and of FEM::Sources (src/fem/sources.cpp:27-75).
 * Patterns are ports x count, column-major (the reference's Matrix<int>). */
typedef struct mpf_eit_desc {
    int32_t n_nodes;
    int32_t n_elements;
    const double* nodes;        /* n x 2 row-major */
    const int32_t* elements;    /* e x 3 row-major */
    const int32_t* edges;       /* edge table from mpf_mesh_edges, n_edges x 2 */
    int32_t n_edges;
    int32_t ports;
    const int32_t* port_edges;  /* ports x port_edges_cap row-major, -1 padded */
    int32_t port_edges_cap;
    int32_t drive_count;
    int32_t meas_count;
    const double* drive_pattern;  /* ports x drive_count, column-major */
    const double* meas_pattern;   /* ports x meas_count, column-major */
    const double* source_values;  /* drive_count values */
    int32_t source_type;          /* enum mpf_source_type */
    double reference_value;
    int32_t logarithmic;          /* 1: sigma = ref * 10^(v/10) */
    int32_t components;           /* 2.5D harmonics */
    double height;
    double port_height;
    int32_t device;               /* CUDA device ordinal */
    /* 0: the reference's 2.5D Jacobian (stiffness term only, harmonic weight
     *    height*beta_c^2; src/fem/equation.cpp:240-247, src/models/eit.cpp:180-205);
     * 1: exact derivative of the 2.5D voltages (adds alpha_c * mass, weight beta_c).
     * Identical for a single harmonic. */
    int32_t jacobian_mode;
    /* Electrode model.  0: the reference's gap model -- a port is a set of
     * boundary edges, its current is spread as the integral of the basis
     * functions over the port divided by the port length and its voltage is
     * the mean potential over it (src/fem/equation.cpp:183-215,
     * src/models/eit.cpp:85-94).  z > 0: the complete electrode model with
     * contact impedance z on every port (Somersalo, Cheney and Isaacson,
     * SIAM J. Appl. Math. 52 (1992) 1023-1040): one voltage unknown per
     * electrode, the boundary term (1/z) int_e (u - U_l) v ds in every
     * harmonic, the current injected into the electrode unknowns and the
     * voltages read from them.  Current (open) sources, real parameters and
     * single models only.  The two models are different physics and are
     * never compared with each other. */
    double contact_impedance;
} mpf_eit_desc;

/* Sizes a caller needs to shape its buffers. */
typedef struct mpf_eit_info {
    int32_t n_nodes, n_elements, data_rows;  /* data_rows: padded node count */
    int32_t ports, drive_count, meas_count;
    int32_t drive_cols_pad, meas_cols_pad;   /* pattern dataCols (multiples of 16) */
    int32_t jacobian_rows;                   /* drive_cols_pad * meas_cols_pad */
    int32_t elements_pad;                    /* element count padded to 64 */
    int32_t density, levels;
    int32_t unique_columns;                  /* distinct excitation vectors solved */
    int32_t components, active_components;   /* harmonics with a nonzero excitation */
} mpf_eit_info;

int mpf_eit_create(const mpf_eit_desc* desc, mpf_eit_t* model);
int mpf_eit_destroy(mpf_eit_t model);
int mpf_eit_get_info(mpf_eit_t model, mpf_eit_info* info);

/* Options of the iterative forward solve. */
typedef struct mpf_solve_opts {
    double tol;            /* relative residual of every system (per right-hand side) */
    int32_t max_iter;      /* 0: 10 * n_nodes, the reference default */
    double refine_tol;     /* > 0: FP64-residual iterative refinement to this level */
    int32_t max_refine;    /* outer refinement steps (default 6) */
    int32_t warm_start;    /* 1: start from the fields left by the previous call (same frame
                            *    count); 2: start every frame from the fields of the
                            *    homogeneous distribution (solved once per model) */
    int32_t check_every;   /* iterations between host convergence checks (default 16) */
    /* 0: Jacobi (the reference's preconditioner::diagonal,
     *    src/numeric/preconditioner.cpp:59-76);
     * 1: two-level -- Jacobi plus an exact coarse correction on aggregates of
     *    64 consecutive (Morton-ordered) nodes, M^-1 = D^-1 + P (P^T A P)^-1 P^T.
     *    Same solutions, fewer iterations; needs <= 64 distinct excitation
     *    columns and <= 32768 nodes, otherwise Jacobi is used. */
    int32_t preconditioner;
    /* 0: conjugate gradient (numeric::ConjugateGradient,
     *    src/numeric/conjugate_gradient.cpp:61-161);
     * 1: BiCGSTAB (numeric::BiCGSTAB, src/numeric/bicgstab.cpp:83-193),
     *    right-preconditioned with Jacobi, each right-hand side stopped at
     *    |r| <= tol |b|; the Neumann harmonic is iterated with the same
     *    c' 1 1^T term as the CG, so both return the same fields.  Needs the
     *    Jacobi preconditioner (preconditioner = 1 is ignored). */
    int32_t solver;
    /* Factor of J J^T + mu I in the Gauss-Newton update (mpf_gn_step,
     * mpf_gn_solve, mpf_gn_solve_learned); the solve of
     * src/solver/inverse.cpp:213-238 is a dense CG on J^T J, both give the
     * regularised update:
     * 0: FP64 Cholesky (default);
     * 1: Cholesky in FP32 arithmetic (a cluster of up to 4 CTAs per frame,
     *    3.9 ms for 32 frames of 1024 against 12.3 ms in FP64) with FP64
     *    iterative refinement to 1e-10 against the FP64 matrix; a frame whose
     *    FP32 factor breaks down or whose refinement stalls falls back to
     *    option 0.  The refinement's triangular solves (2.2 ms per step for 32
     *    frames) make it slower than option 0 on the 1024-row system. */
    int32_t gn_factor;
    /* mpf_gn_solve_learned only: CG tolerance of the solve at the network's
     * prediction, whose only use is the accept / reject decision (0 or <= tol:
     * that solve runs at tol).  A frame whose data residual at accept_tol is
     * <= target (1 - accept_margin) is accepted on it; every other frame
     * continues from its fields to tol (the assembled systems and the coarse
     * space are kept) and is decided on its full-tolerance residual, as
     * without the option.  accept_margin (default 0.1 when 0) covers the
     * difference between the two residuals. */
    double accept_tol;
    double accept_margin;
} mpf_solve_opts;

typedef struct mpf_solve_stats {
    int32_t iterations;        /* CG iterations of the slowest system, summed over refinements */
    int32_t refinements;
    int32_t not_converged;     /* systems that hit max_iter */
    double max_rel_residual;   /* largest final relative residual (FP64 when refining) */
    double seconds;            /* host wall time of the call (synchronised) */
} mpf_solve_stats;

/* sigma -> stiffness S and mass R slot values in the reference ELL layout
 * (dataRows x 32 row-major per frame), i.e. Equation::update's two
 * updateMatrix launches (src/fem/equation.cpp:261-274,
 * src/fem/equation_kernel.cu:60-82).  gamma: frames x n_elements.
 * s_values / r_values: frames x data_rows x 32 floats. */
int mpf_eit_assemble(mpf_eit_t model, int32_t frames, const float* gamma, float* s_values,
                     float* r_values, mpf_stream_t stream);

/* Forward solve of all frames x harmonics x excitations in one batch:
 * EIT::solve (src/models/eit.cpp:139-213) for current sources.
 *   gamma:    frames x n_elements (device, float)
 *   voltages: frames x meas_count x drive_count, column-major per frame
 *             (the reference's result Matrix, Mm x Md) or NULL
 *   jacobian: frames x jacobian_rows x n_elements, column-major per frame
 *             (the reference's jacobian Matrix) or NULL
 * Synchronises the stream (convergence is checked on the host every
 * opts->check_every iterations). */
int mpf_eit_forward(mpf_eit_t model, int32_t frames, const float* gamma, float* voltages,
                    float* jacobian, const mpf_solve_opts* opts, mpf_solve_stats* stats,
                    mpf_stream_t stream);

/* Potential fields of the last forward solve in the reference layout
 * (EIT::fields): component c of frame f as a data_rows x (drive+meas)
 * column-major float matrix.  fields: frames x components x data_rows x
 * (drive_count + meas_count). */
int mpf_eit_fields(mpf_eit_t model, int32_t frames, float* fields, mpf_stream_t stream);

/* Complex potential fields of the last mpf_eit_forward_complex call, same
 * layout as mpf_eit_fields with interleaved (re, im) float pairs: fields
 * holds frames x components x data_rows x (drive_count + meas_count)
 * complex values (the reference's EIT::fields of its complex
 * instantiations, src/models/eit.cpp:152-180). */
int mpf_eit_fields_complex(mpf_eit_t model, int32_t frames, float* fields, mpf_stream_t stream);

/* EIT::solve for complex material values: the reference's
 * models::EIT<..., FEM::Equation<thrust::complex<float>, ...>> instantiations
 * (src/models/eit.cpp:289-304).  p(gamma) = ref * gamma or
 * ref * exp(ln(10) gamma / 10) with complex gamma
 * (src/fem/equation_kernel.cu:35-43; a complex reference value is expressed
 * through gamma), complex S and R, BiCGSTAB over complex vectors with the
 * reference's inner product sum a conj(b) (src/numeric/matrix_kernel.cu:
 * 404-413), Jacobi-preconditioned, each right-hand side stopped at
 * |r| <= tol |b|, FP32 with FP64 inner products.
 *   gamma:    device, frames x n_elements complex (re, im interleaved)
 *   voltages: device, frames x (Mm x Md column-major) complex, interleaved
 *   jacobian: device, frames x (jacobian_rows x n_elements column-major)
 *             complex, interleaved, or NULL: calcJacobian's bilinear form
 *             with complex fields and complex p'(gamma)
 *             (src/fem/equation_kernel.cu:197-245)
 * Cold start only; MPF_ENOTSUP for refine_tol > 0, warm_start != 0, voltage
 * (fixed) sources or more than 64 unique excitations.  Synchronises
 * `stream`. */
int mpf_eit_forward_complex(mpf_eit_t model, int32_t frames, const float* gamma, float* voltages, float* jacobian,
                            const mpf_solve_opts* opts, mpf_solve_stats* stats, mpf_stream_t stream);

/* ======================================================================== */
/* Regularised Gauss-Newton                                                  */
/* ======================================================================== */

/* One Gauss-Newton step per frame, solveAbsolute (src/solver/solver.cpp:196-225)
 * with Inverse::updateJacobian + solve (src/solver/inverse.cpp:60-238) for
 * R = I, in dual form:
 *   dgamma = J^T (J J^T + mu I)^{-1} (v_meas - V(gamma)),  mu = (ref*lambda)^2
 * J J^T from split hi+lo BF16 tcgen05 products, FP64 Cholesky.
 *   gamma:     frames x n_elements, updated in place
 *   v_meas:    frames x meas_count x drive_count (column-major per frame)
 *   residual:  frames doubles, ||v_meas - V(gamma_in)|| / ||v_meas|| (or NULL)
 * Synchronises the stream. */
int mpf_gn_step(mpf_eit_t model, int32_t frames, float* gamma, const float* v_meas, double lambda,
                const mpf_solve_opts* opts, double* residual, mpf_solve_stats* stats,
                mpf_stream_t stream);

typedef struct mpf_gn_stats {
    int32_t gn_iterations;    /* Gauss-Newton updates applied (slowest frame) */
    int32_t cg_iterations;    /* CG iterations summed over the forward solves (slowest group) */
    int32_t frames_converged; /* frames whose residual reached the target */
    double seconds;           /* host wall time of the call (synchronised) */
    int32_t solves_fp32;      /* frame updates solved by the FP32 factor with FP64 refinement */
    int32_t solves_fp64;      /* frame updates solved by the FP64 factor (gn_factor 1, or the fallback) */
    int32_t accepted_loose;   /* mpf_gn_solve_learned: frames decided on the accept_tol solve */
} mpf_gn_stats;

/* Batched Gauss-Newton reconstruction: repeats mpf_gn_step on every frame
 * whose relative data residual ||v_meas - V(gamma)|| / ||v_meas|| is above
 * `target`, for at most max_gn_iters updates; frames that reach the target
 * are frozen.  The reference leaves this outer loop to its caller
 * (src/solver/solver.cpp:196-225 is one step).  Forward solves after the
 * first start from the previous fields.  A frame whose J J^T + mu I is not
 * positive definite also in FP64, or whose update leaves the forward model's
 * range (a non-finite value, |gamma| > 100 dB logarithmic, gamma <= 0
 * linear), keeps its last gamma and is frozen unconverged; the other frames
 * go on (mpf_gn_step reports a breakdown as MPF_EBREAKDOWN instead).
 *   iterations: host, frames ints (updates per frame) or NULL
 *   residual:   host, frames doubles (final residual per frame) or NULL */
int mpf_gn_solve(mpf_eit_t model, int32_t frames, float* gamma, const float* v_meas, double lambda,
                 double target, int32_t max_gn_iters, const mpf_solve_opts* opts, int32_t* iterations,
                 double* residual, mpf_gn_stats* stats, mpf_stream_t stream);

/* Regulariser of the inverse step: solver::Inverse::RegularizationType
 * (include/mpflow/solver/inverse.h:31-35). */
enum mpf_regularization { MPF_REG_IDENTITY = 0, MPF_REG_NOSER = 1, MPF_REG_LAPLACIAN = 2 };

/* One regularised inverse step, solver::Inverse::updateJacobian + solve
 * (src/solver/inverse.cpp:60-238):
 *   (J^T J + (ref * factor)^2 R) result = J^T (measurement - calculation)
 * for `images` right-hand sides (parallelImages), R = I, diag(J^T J) (NOSER)
 * or L^T L with the reference's edge-length Laplacian.  R = I is solved in
 * its dual form for any mesh size; NOSER and Laplacian assemble the E x E
 * system and need n_elements <= 6144 (MPF_ENOTSUP beyond).  Exact FP64
 * Cholesky solve where the reference runs a dense CG.  Synchronises.
 *   jacobian:    device, reference layout (column-major jacobian_rows x E),
 *                e.g. the output of mpf_eit_forward
 *   calculation, measurement: device, images x (meas_count * drive_count),
 *                each image column-major meas_count x drive_count
 *   result:      device, images x n_elements */
int mpf_inverse_solve(mpf_eit_t model, int32_t regularization, double factor, int32_t images,
                      const float* jacobian, const float* calculation, const float* measurement,
                      float* result, mpf_stream_t stream);

/* Kernel timing hook for the FEM kernels: after a forward solve of `gamma`,
 * times `reps` launches each of the assembly (S, R slot values of all
 * frames) and of the Jacobian (split-BF16 J of all frames) with CUDA events
 * on `stream`; ms[2] mean time of one launch, bytes[2] its algorithmic bytes.
 * No reference counterpart (measurement support).  Synchronises. */
int mpf_eit_profile_fem(mpf_eit_t model, int32_t frames, const float* gamma, int32_t reps, double* ms,
                        double* bytes, mpf_stream_t stream);

/* Kernel timing hook: runs `reps` CG iterations on the systems of `gamma`
 * and reports, for the SpMM, update and direction kernels, the mean CUDA-
 * event time of one launch (ms[3]) and its algorithmic bytes (bytes[3]).
 * No reference counterpart (measurement support). */
int mpf_eit_profile_cg(mpf_eit_t model, int32_t frames, const float* gamma, int32_t reps, double* ms,
                       double* bytes, mpf_stream_t stream);

/* Launch and graph overhead of the CG loop on the systems of `gamma`
 * (tolerance 0, every group iterating): ms[0] the per-iteration time of the
 * loop as a solve runs it (CUDA graphs of 16 iterations with the host
 * convergence check between graphs), timed by CUDA events around `graphs`
 * graphs; ms[1] the per-iteration sum of the same kernels launched one at a
 * time between CUDA events; ms[2] the host wall clock per iteration of the
 * loop.  1 - ms[1] / ms[0] is the share of the loop spent outside the
 * kernels.  The reference launches each iteration's kernels from the host
 * (src/numeric/conjugate_gradient.cpp:111-157).  Synchronises. */
int mpf_eit_profile_cg_loop(mpf_eit_t model, int32_t frames, const float* gamma, int32_t graphs, double* ms,
                            mpf_stream_t stream);

/* Device-time breakdown of the model's forward and Gauss-Newton calls by
 * phase.  While enabled, the library records a CUDA event on the call's
 * stream at every change of phase and attributes the time between
 * consecutive events to the phase that ran there, so the phases of a call add
 * up to its device time from the first mark to the last (gaps in which the
 * device waits for the host count toward the phase that follows them).
 * enable = 1 starts (and clears) the accumulation, 0 stops it, -1 leaves it
 * as it is; ms[min(cap, MPF_PHASES)] receives the milliseconds accumulated per
 * phase (indices MPF_PHASE_*) and *calls the top-level calls timed.
 * No reference counterpart (measurement support). */
#define MPF_PHASES 11
#define MPF_PHASE_ASSEMBLY 0    /* S, R slot values (and FP64 copies, Dirichlet rows) */
#define MPF_PHASE_CG_SETUP 1    /* launch-shape autotuning, coarse-space factor and inverse */
#define MPF_PHASE_CG 2          /* Krylov iterations, FP64 refinement, warm-start copies */
#define MPF_PHASE_VOLTAGES 3    /* electrode voltages and data residuals */
#define MPF_PHASE_JACOBIAN 4
#define MPF_PHASE_GRAM 5        /* J J^T + mu I (tensor-core split-BF16, FP64 fallback) */
#define MPF_PHASE_CHOLESKY 6    /* FP64 factor and triangular solves */
#define MPF_PHASE_UPDATE 7      /* gamma += J^T w, range check, undo of diverged frames */
#define MPF_PHASE_NETWORK 8     /* learned start: network forward pass */
#define MPF_PHASE_PRIOR 9       /* learned start: network input and linear prior */
#define MPF_PHASE_HOST 10       /* host decisions between device work (masks, convergence checks) */
int mpf_eit_phase_times(mpf_eit_t model, int32_t enable, double* ms, int32_t cap, int64_t* calls);

/* CG iterations of every (frame, harmonic) group in the last inner solve of
 * the last forward call, group g = frame * active_components + harmonic.
 * Writes min(count, cap) entries; *count receives the group count.  The
 * reference returns one summed count (src/models/eit.cpp:207-210). */
int mpf_eit_group_iterations(mpf_eit_t model, int32_t* iterations, int32_t cap, int32_t* count);

/* Launch shapes of the CG SpMM, update and direction kernels.  Shape
 * code = 3 * i + k + 9 * t (+ 36 * u for the SpMM) runs {4, 2, 1}[i] floats
 * per lane, keeps {1, 2, 4}[k] row steps in flight per warp and walks 2^t
 * (t = 0..3) tiles of 128 rows per block; u = 1 stages each tile's ELL slots
 * in shared memory one tile ahead (SpMM codes 0..71, others 0..35).  By default the first cold solve with a given frame
 * count times every shape on the model's own systems and keeps the fastest
 * of each kernel (the reference's launch shape is fixed: src/numeric/
 * sparse_matrix.cpp:262-288).
 *   set: host, 3 ints, each a shape code or -1 (autotune), or NULL to leave
 *        as is
 *   get: host, 3 ints receiving the codes a solve with `frames` frames uses,
 *        or NULL
 * Fails with MPF_EINVAL for a shape that the right-hand-side width does not
 * allow.  No reference counterpart. */
int mpf_eit_cg_variants(mpf_eit_t model, const int32_t* set, int32_t frames, int32_t* get);

/* ======================================================================== */
/* Dense matrix operations (numeric::Matrix)                                 */
/* ======================================================================== */

/* Device operations of the reference's column-major dense Matrix
 * (src/numeric/matrix.cpp, kernels src/numeric/matrix_kernel.cu:35-631) on
 * rows x cols FP32 matrices with leading dimension ld (>= rows, the
 * reference's dataRows).  op: 0 setEye (C = I), 1 diag (C = diagonal of A),
 * 2 add scalar (C = A + scalar), 3 add (C = A + B), 4 scalarMultiply
 * (C = scalar A), 5 elementwiseMultiply (C = A .* B), 6 elementwiseDivision
 * (C = A ./ B, 0 where B = 0).  C may alias A. */
int mpf_matrix_elementwise(int32_t op, int32_t rows, int32_t cols, const float* A, const float* B, float* C,
                           int32_t ld, float scalar, mpf_stream_t stream);

/* count scalars on the device between the reference's wider data types and
 * the library's FP32 (direction 0: double -> float, 1: float -> double; a
 * complex value is two scalars).  The C++ facade converts the material,
 * voltages, Jacobian and fields of its double and complex<double>
 * instantiations (src/models/eit.cpp:273-304 instantiates those natively)
 * with this, stream-ordered and without host copies. */
int mpf_convert_values(int32_t direction, int64_t count, const void* src, void* dst, mpf_stream_t stream);

/* Column reductions into row 0 of each column of result (leading dimension
 * ldr), as Matrix::sum / vectorDotProduct / min / max leave them
 * (src/numeric/matrix.cpp:455-660): op 0 sum, 1 dot of A and B, 2 min, 3 max; FP64
 * accumulation in a fixed order. */
int mpf_matrix_column_reduce(int32_t op, int32_t rows, int32_t cols, const float* A, const float* B, int32_t ld,
                             float* result, int32_t ldr, mpf_stream_t stream);

/* Matrix::multiply's cuBLAS GEMM (src/numeric/matrix.cpp:298-332): C (m x n) =
 * op(A) op(B) with op(X) = X (trans 0) or X^T (trans 1), column-major,
 * FP32 on a tiled kernel of this library. */
int mpf_matrix_multiply(int32_t trans_a, int32_t trans_b, int32_t m, int32_t n, int32_t k, const float* A,
                        int32_t lda, const float* B, int32_t ldb, float* C, int32_t ldc, mpf_stream_t stream);

/* ======================================================================== */
/* Sparse matrices and Krylov solvers on a caller's matrix                   */
/* ======================================================================== */

/* numeric::SparseMatrix (include/mpflow/numeric/sparse_matrix.h:30-80) built
 * from the reference ELL layout: values and column_ids are DEVICE arrays of
 * data_rows(rows) x 32 (row-major, 0xFFFFFFFF padding), as
 * SparseMatrix::deviceValues / deviceColumnIds; density = used slots per row
 * (at most 32, MPF_EFULL otherwise).  The library keeps its own copy. */
typedef struct mpf_sparse* mpf_sparse_t;
int mpf_sparse_create(int32_t rows, const float* values, const uint32_t* column_ids, uint32_t density,
                      mpf_sparse_t* matrix);
int mpf_sparse_destroy(mpf_sparse_t matrix);

/* SparseMatrix::multiply (src/numeric/sparse_matrix.cpp:262-288): y = A x for
 * `cols` column-major columns (device, leading dimensions ldx, ldy >= rows). */
int mpf_sparse_multiply(mpf_sparse_t matrix, const float* x, int32_t ldx, int32_t cols, float* y, int32_t ldy,
                        mpf_stream_t stream);

/* ConjugateGradient::solve / BiCGSTAB::solve (src/numeric/conjugate_gradient.cpp:
 * 61-161, src/numeric/bicgstab.cpp:83-193) on every column of b at once,
 * each column an independent system with its own scalars and convergence
 * mask; x (device, column-major, ldx) is the initial guess and receives the
 * solution.  solver: 0 CG, 1 BiCGSTAB; always Jacobi-preconditioned (the
 * reference's KInv = preconditioner::diagonal).  dc_free solves
 * (A + 1 1^T) x = b as the reference's iteration (its initial residual adds
 * +sum(x) instead, src/numeric/conjugate_gradient.cpp:86-89; the same for a
 * zero start).  max_iter <= 0: 10 * rows; tol <= 0: float epsilon, the
 * reference's level.  *iterations: slowest column.  MPF_ENOCONV when a
 * column hits max_iter (the reference returns silently).  Synchronises. */
int mpf_sparse_solve(mpf_sparse_t matrix, int32_t solver, const float* b, int32_t ldb, float* x, int32_t ldx,
                     int32_t cols, int32_t max_iter, double tol, int32_t dc_free, int32_t* iterations,
                     mpf_stream_t stream);

/* ======================================================================== */
/* Batches of uneven meshes                                                  */
/* ======================================================================== */

/* Forward solves of several models -- meshes of different size and electrode
 * count sharing one harmonic set (components, height) -- as independent
 * systems in the same CG launches: one launch per kernel and right-hand-side
 * width (16, 32, 64 or 128 unique excitations) covers every (mesh, frame,
 * harmonic) group, each with its own scalars and convergence mask.  The
 * reference solves one EIT model at a time (EIT::solve,
 * src/models/eit.cpp:139-213); calling it once per mesh gives the same
 * voltages.  The models must outlive the batch; they stay usable on their
 * own.  Fails with MPF_ENOTSUP for voltage (fixed) sources and MPF_EINVAL for
 * models on different devices or with different harmonic sets. */
typedef struct mpf_batch* mpf_batch_t;
int mpf_batch_create(const mpf_eit_t* models, int32_t count, mpf_batch_t* batch);
int mpf_batch_destroy(mpf_batch_t batch);

/* EIT::solve for `frames` frames of every model.  gamma[i]: device,
 * frames x n_elements(i); voltages[i]: device, frames x Mm(i) x Md(i), each
 * frame column-major (as mpf_eit_forward).  Both are host arrays of `count`
 * device pointers.  Cold start, FP32, CG (Jacobi or, with
 * opts->preconditioner = 1, the two-level preconditioner on every mesh's own
 * coarse space) or BiCGSTAB (Jacobi); MPF_ENOTSUP for refine_tol > 0 or
 * warm_start != 0.  CG launch shapes are autotuned per width class at the
 * first call with a frame count.
 * Synchronises `stream`.  stats->iterations: slowest group. */
int mpf_batch_forward(mpf_batch_t batch, int32_t frames, const float* const* gamma, float* const* voltages,
                      const mpf_solve_opts* opts, mpf_solve_stats* stats, mpf_stream_t stream);

/* CG iterations of every group of the last mpf_batch_forward, ordered
 * [model][frame][active harmonic]; writes min(count, cap) entries. */
int mpf_batch_iterations(mpf_batch_t batch, int32_t* iterations, int32_t cap, int32_t* count);

/* Device time of the last call's Krylov solve (initialisation and
 * iterations, CUDA events on its stream) and the algorithmic bytes its
 * iterations moved: per iteration and group nnz * 12 + 10 * K * n * 4 +
 * 4 * n * 4 for CG (SpMM, update and direction passes; K unique excitations,
 * n nodes of the group's mesh; two-level: + ncPad^2 * 4 + 3 * ncPad * K * 4
 * for the coarse product), 2 * nnz * 12 + 21 * K * n * 4 + 6 * n * 4 for
 * BiCGSTAB.  No reference counterpart (measurement support). */
int mpf_batch_cg_stats(mpf_batch_t batch, double* cg_ms, double* cg_bytes);

/* Launch shapes of the batch's CG kernels (codes as mpf_eit_cg_variants):
 * set (3 codes or -1, or NULL) applies to every width class; get receives
 * 3 codes per width class (ascending width, at most cap entries) used with
 * `frames` frames; *classes receives the number of width classes. */
int mpf_batch_cg_variants(mpf_batch_t batch, const int32_t* set, int32_t frames, int32_t* get, int32_t cap,
                          int32_t* classes);

/* ======================================================================== */
/* Dense building blocks                                                     */
/* ======================================================================== */

/* C = A A^T for batch row-major FP32 matrices A (rows x cols, leading
 * dimension lda >= cols, lda % 8 == 0) with split hi+lo BF16 products
 * (hi.hi + hi.lo + lo.hi) on the tcgen05 tensor cores, FP32 accumulation;
 * C is rows x rows row-major (symmetric).  rows % 128 == 0, cols % 64 == 0.
 * The replaced reference product is the cuBLAS J^T J of
 * src/solver/inverse.cpp:136-156 (taken here in its dual orientation).
 * Every pipeline wait inside the kernel is bounded (2 s); a wait that gives
 * up makes the call return MPF_ETIMEOUT, and C is then undefined. */
int mpf_gram_split_bf16(int32_t batch, int32_t rows, int32_t cols, const float* A, int32_t lda,
                        float* C, mpf_stream_t stream);

/* mpf_gram_split_bf16 without any device allocation.  No counterpart in the
 * reference.  For callers that cannot allocate device memory after start-up
 * (a real-time loop that must not stall on cudaMalloc's implicit device
 * synchronisation, or a host framework whose allocator owns the device): the
 * BF16 hi/lo copies, split-K partials and abort flag live in fixed device
 * arrays inside the library (12 MB per GPU that loads it, kept until exit)
 * instead of per-call buffers.  Same arguments and result as
 * mpf_gram_split_bf16; limits batch*rows*lda <= 2,097,152 elements and a
 * split-K workspace <= 1,048,576 floats, larger requests return MPF_EINVAL.
 * All calls share the arrays: calls that overlap on the GPU race and corrupt
 * each other's results.  Every call reads its abort flag back to the host
 * and synchronises the stream, so the call cannot be captured into a CUDA
 * graph: issue it on a stream that is not capturing. */
int mpf_gram_split_bf16_noalloc(int32_t batch, int32_t rows, int32_t cols, const float* A, int32_t lda,
                                float* C, mpf_stream_t stream);

/* Measurement hook: device time of the GN step's J J^T (split-BF16 tcgen05
 * Gram of batch row-major rows x cols operands plus its split-K reduction
 * into FP64 with a diagonal shift) on synthetic operands the call allocates,
 * averaged over `reps` launches timed with CUDA events on `stream`.
 * rows % 128 == 0, cols % 64 == 0.  No reference counterpart (measurement
 * support).  Synchronises. */
int mpf_profile_gram(int32_t batch, int32_t rows, int32_t cols, int32_t reps, double* ms_per_launch,
                     mpf_stream_t stream);

/* Batched FP64 Cholesky solve of (A + shift I) X = B, A n x n symmetric
 * (row-major == column-major), B n x nrhs column-major, per batch entry.
 * A is overwritten by its factor.  info[batch] (device ints) receives 0 or
 * the 1-based index of the first non-positive pivot.  n must be a multiple
 * of 32 and at most 24576.  Replaces the dense CG of Inverse::solve
 * (src/solver/inverse.cpp:213-238). */
int mpf_cholesky_solve_f64(int32_t batch, int32_t n, double* A, double shift, double* B,
                           int32_t nrhs, int32_t* info, mpf_stream_t stream);

/* ======================================================================== */
/* Learned Gauss-Newton warm start.  No reference counterpart: the reference */
/* starts every reconstruction from the homogeneous distribution            */
/* (src/solver/solver.cpp:196-225).                                          */
/* ======================================================================== */

typedef struct mpf_mlp* mpf_mlp_t;

/* Multilayer perceptron in -> hidden1 -> hidden2 -> out with GELU on the
 * hidden layers, BF16 weights and activations on the tcgen05 tensor cores
 * with FP32 accumulation, FP32 master weights.  Widths are multiples of 128.
 * Weights are LeCun-uniform from `seed`, biases zero.  Synchronises. */
int mpf_mlp_create(int32_t in, int32_t hidden1, int32_t hidden2, int32_t out, uint64_t seed,
                   int32_t device, mpf_mlp_t* net);
int mpf_mlp_destroy(mpf_mlp_t net);

/* Layout of the flat FP32 parameter array: offsets[7] = {W1, b1, W2, b2, W3,
 * b3, total}; each W row-major (outputs x inputs). */
int mpf_mlp_layout(mpf_mlp_t net, int64_t* offsets);

/* y (device, batch x ldy) = net(x) for x (device, batch x in FP32); the
 * first min(ldy, out) outputs of each row are written.  Synchronises. */
int mpf_mlp_forward(mpf_mlp_t net, int32_t batch, const float* x, float* y, int32_t ldy,
                    mpf_stream_t stream);

/* Forward and backward pass of the loss
 *   (1 / (batch * valid)) sum_b sum_{j < valid} (y[b][j] - target[b][j])^2
 * (target: device, batch x ldt) into the network's gradient array.  *loss
 * (host) receives the loss when non-NULL, which synchronises the stream. */
int mpf_mlp_backward(mpf_mlp_t net, int32_t batch, const float* x, const float* target, int32_t ldt,
                     int32_t valid, double* loss, mpf_stream_t stream);

/* One Adam step from the current gradients; weight_decay is decoupled and
 * applies to the weight matrices only. */
int mpf_mlp_adam(mpf_mlp_t net, float lr, float beta1, float beta2, float eps, float weight_decay,
                 mpf_stream_t stream);

/* One training step: mpf_mlp_backward on batch rows gathered by index
 * (batch row b is row rows[b] of x, leading dimension ldx >= in, and of
 * target, leading dimension ldt; rows = NULL takes rows 0..batch-1), then
 * mpf_mlp_adam.  Same update, bit for bit, as the two calls on gathered
 * copies, without the copies; the last layer's weight gradient is not
 * stored (its Adam step runs in the epilogue of the tensor-core product that
 * forms it), so the gradient array afterwards holds every gradient but that
 * one.  rows is a device array of batch indices. */
int mpf_mlp_train_step(mpf_mlp_t net, int32_t batch, const float* x, int32_t ldx, const int32_t* rows,
                       const float* target, int32_t ldt, int32_t valid, float lr, float beta1, float beta2,
                       float eps, float weight_decay, double* loss, mpf_stream_t stream);

/* Device buffer of offsets[6] floats <-> network: which = 0 reads the
 * parameters, 1 writes them (and resets the Adam state), 2 reads the
 * gradients of the last mpf_mlp_backward. */
int mpf_mlp_params(mpf_mlp_t net, float* buffer, int32_t which, mpf_stream_t stream);

/* Network input of the learned warm start, x[f][i] = (v_meas[f][i] - V0[i])
 * / rms(V0) for the meas_count x drive_count voltages of each frame, V0 the
 * voltages of the homogeneous distribution (gamma = 0 logarithmic, 1 linear;
 * solved once per model).  v_meas and x: device, frames x (meas_count *
 * drive_count) FP32. */
int mpf_eit_learned_input(mpf_eit_t model, int32_t frames, const float* v_meas, float* x,
                          mpf_stream_t stream);

/* Complex regularised inverse step, solver::Inverse<thrust::complex<float>>
 * (src/solver/inverse.cpp:60-238, instantiated at :243):
 *   (J^T J + (ref * factor)^2 R) result = J^T (measurement - calculation)
 * with the plain (unconjugated) transpose of the reference's CUBLAS_OP_T
 * products, R as in mpf_inverse_solve (identity in dual form for any mesh,
 * NOSER and Laplacian on the E x E system for n_elements <= 6144).  The Gram
 * is formed in FP64 from the FP32 J and factored as a complex symmetric
 * L L^T in FP64 without pivoting where the reference runs a dense CG;
 * MPF_EBREAKDOWN on a zero pivot.  Complex arrays hold interleaved (re, im)
 * floats (thrust::complex<float>); shapes as in mpf_inverse_solve, e.g. the
 * jacobian output of mpf_eit_forward_complex.  Synchronises. */
int mpf_inverse_solve_complex(mpf_eit_t model, int32_t regularization, double factor, int32_t images,
                              const float* jacobian, const float* calculation, const float* measurement,
                              float* result, mpf_stream_t stream);

/* Linear prior of the learned start: the first Gauss-Newton update from the
 * homogeneous distribution gamma_h, which is linear in the network input x,
 *   prior(x) = gamma_h + J0^T (J0 J0^T + mu I)^-1 x / rms-scale,
 * mu = (referenceValue lambda)^2 as in mpf_gn_step, J0 the FP32 Jacobian at
 * gamma_h with the Gram and its Cholesky factor in FP64 (the fixed part of
 * Solver::solveAbsolute's first iteration, src/solver/solver.cpp:196-225,
 * taken once per model).  Held by the model as split-BF16 operands of an
 * n_elements x (meas_count * drive_count) matrix (hi, lo parts), applied on
 * the tensor cores as hi.hi + lo.hi + hi.lo with FP32 accumulation (about
 * FP32 accuracy); lambda = 0 removes it.  While a prior is set,
 * mpf_gn_solve_learned starts from prior(x) + net(x), so the network learns
 * the correction to the linear step.  Synchronises. */
int mpf_eit_learned_prior(mpf_eit_t model, double lambda, mpf_stream_t stream);

/* out (device, frames x ldo, ldo >= n_elements) = prior(x) (mode 0),
 * out += prior(x) (mode 1) or out -= prior(x) (mode -1); x device, frames x
 * (meas_count * drive_count).  MPF_EINVAL when no prior is set.
 * Synchronises (reads the product's abort flag). */
int mpf_eit_learned_prior_apply(mpf_eit_t model, int32_t frames, const float* x, float* out, int32_t ldo,
                                int32_t mode, mpf_stream_t stream);

/* Gauss-Newton from a learned start.  gamma (device, frames x n_elements,
 * output) starts as the network's prediction for each frame's voltages (plus
 * the linear prior when one is set, mpf_eit_learned_prior); a
 * frame keeps it only if its relative data residual there is below the
 * homogeneous start's, otherwise it restarts from the homogeneous
 * distribution (accepted[f] = 0).  Then mpf_gn_solve iterations to `target`.
 * The network maps meas_count * drive_count inputs to >= n_elements outputs.
 *   iterations, residual, accepted: host, frames entries each, or NULL.
 * Synchronises. */
int mpf_gn_solve_learned(mpf_eit_t model, mpf_mlp_t net, int32_t frames, float* gamma,
                         const float* v_meas, double lambda, double target, int32_t max_gn_iters,
                         const mpf_solve_opts* opts, int32_t* iterations, double* residual,
                         int32_t* accepted, mpf_gn_stats* stats, mpf_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* MPFLOW_GB300_H */
