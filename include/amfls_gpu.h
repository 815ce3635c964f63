/* amfls_gpu.h - C ABI of the GB300-native AMFLS least-squares solver.
 *
 * Drop-in boundary for the reference's AMFLS hot path
 * (doloMing/amfls_solver).  Every entry point takes plain pointers and sizes;
 * matrix and vector arguments named d_* are CUDA device pointers, `stream` is
 * a cudaStream_t passed as void* (NULL = the legacy default stream).  All
 * functions return AMFLS_GPU_OK (0) or an error code; amfls_gpu_last_error()
 * gives the message of the calling thread's last failure.  Numerical outcomes
 * are never errors: they are reported through status / stop_reason with the
 * reference's integer values.
 *
 * Reference interfaces replaced (paths relative to the reference repository):
 *   MatrixOperator contract ......... include/amfls/matrix_operator.hpp:29-89
 *   SparseCsrOperator ............... src/algorithms/mathematics/operators/sparse_csr_operator.hpp:13-58
 *   AmflsOptions / solve_amfls ...... include/amfls/amfls.hpp:10-25
 *   FixedRbgkOptions / solve_fixed_rbgk include/amfls/fixed_rbgk.hpp:8-25
 *   LeastSquaresResult / statuses ... include/amfls/least_squares_result.hpp:8-229
 *   result tensor layout ............ bindings/torch/result_tensors.hpp:12-156
 */
#ifndef AMFLS_GPU_H
#define AMFLS_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    AMFLS_GPU_OK = 0,
    AMFLS_GPU_INVALID_ARGUMENT = 1, /* std::invalid_argument in the reference */
    AMFLS_GPU_LENGTH_ERROR = 2,     /* std::length_error / overflow_error */
    AMFLS_GPU_LOGIC_ERROR = 3,      /* std::logic_error */
    AMFLS_GPU_CUDA_ERROR = 4,       /* a CUDA runtime call failed */
    AMFLS_GPU_RUNTIME_ERROR = 5     /* any other failure */
};

/* SolverStatus (least_squares_result.hpp:8-14) */
enum {
    AMFLS_STATUS_SUCCESS = 0,
    AMFLS_STATUS_WORK_LIMIT = 1,
    AMFLS_STATUS_BASIS_LIMIT = 2,
    AMFLS_STATUS_PRECISION_LIMIT = 3,
    AMFLS_STATUS_NUMERICAL_BREAKDOWN = 4
};

/* Widths of the packed result arrays (result_tensors.hpp:12-16). */
#define AMFLS_GPU_METRICS 21
#define AMFLS_GPU_COUNTERS 36
#define AMFLS_GPU_TIMINGS 9
#define AMFLS_GPU_TRACE_FLOAT 29
#define AMFLS_GPU_TRACE_INT 4

typedef struct amfls_gpu_operator amfls_gpu_operator;

/* MatrixOperatorValidationErrorModel (matrix_operator.hpp:21-27). */
typedef struct {
    double operator_norm_upper_bound;
    double operator_norm_lower_bound;
    long long apply_rounding_steps;
    long long apply_transpose_rounding_steps;
} amfls_gpu_validation_error_model;

/* AmflsOptions (amfls.hpp:10-20) and FixedRbgkOptions (fixed_rbgk.hpp:8-18). */
typedef struct {
    double regularization;       /* lambda >= 0 */
    double tolerance;            /* (0, 1) */
    double failure_probability;  /* (0, 1); validated, does not change the algorithm */
    int maximum_epochs;          /* 0 = default */
    int maximum_basis_size;      /* 0 = min(rows, cols) */
    uint64_t seed;
    uint64_t stream;             /* random stream id (not a CUDA stream) */
    int maximum_depth;           /* 0 = min(rows, cols); fixed RBGK: required > 0 */
    int maximum_auxiliary_width; /* 0 = default */
    int auxiliary_width;         /* fixed RBGK only */
    int stop_early;              /* fixed RBGK only */
    int time_operators;          /* record device times of operator calls (default 1) */
    int use_graphs;              /* run width-one levels as one CUDA graph per checkpoint
                                    interval (default 1); 0 launches the same kernels one by
                                    one, e.g. for per-kernel profiling */
    int reduced_basis;           /* mixed-precision sweeps (default 0; no counterpart in the
                                    reference): 1 (FP32) or 2 (FP16, holding 2^8 v):
                                    width-one levels keep a reduced copy of the right basis V
                                    and run their first reorthogonalisation pass on it (FP32
                                    products, FP64 subtraction), redoing it in FP64 when its
                                    coefficients exceed 1e-3 ||r||; the
                                    recurrence, products, DGKS second pass, projected solve
                                    and validation stay FP64.  V then stays orthogonal to
                                    about FP32 rounding / sqrt(rows), which suits the restart
                                    cycles of amfls_gpu_solve_amfls_mixed; a single solve of
                                    an ill-conditioned problem to FP64 accuracy can stall on
                                    it (reported by the certificate, never a false success).
                                    Costs 4 (FP32) or 2 (FP16) extra bytes per basis element
                                    of device memory.  Any other value makes every solve
                                    entry point return AMFLS_GPU_INVALID_ARGUMENT before any
                                    device work. */
} amfls_gpu_options;

/* LeastSquaresResult, packed like the torch binding's tensors. */
typedef struct {
    int rows, cols, iterations, depth, auxiliary_width, basis_rank;
    int status, stop_reason;
    double metrics[AMFLS_GPU_METRICS];
    long long counters[AMFLS_GPU_COUNTERS];
    double timings[AMFLS_GPU_TIMINGS];
    int trace_rows; /* checkpoints evaluated; rows beyond the capacity are dropped */
    long long kernel_launches; /* GPU kernels the solve ran (not part of the reference) */
    long long reduced_basis_levels;    /* levels projected on the reduced copy of V (reduced_basis) */
    long long reduced_basis_fallbacks; /* of those, levels whose projection was redone in FP64 */
} amfls_gpu_result;

/* LsqrOptions (lsqr.hpp:8-12) and LsmrOptions (lsmr.hpp): the same fields. */
typedef struct {
    double regularization;  /* lambda >= 0 (damp^2) */
    double tolerance;       /* (0, 1) */
    int maximum_iterations; /* 0 = min(rows, cols) */
} amfls_gpu_baseline_options;

/* Sets the reference's defaults (amfls.hpp:10-20; fixed_rbgk.hpp:8-18). */
void amfls_gpu_default_options(amfls_gpu_options* options);

/* Sets LsqrOptions' / LsmrOptions' defaults (lambda 0, tol 1e-8, 0 iterations). */
void amfls_gpu_default_baseline_options(amfls_gpu_baseline_options* options);

/* Message of the calling thread's last error ("" if none). */
const char* amfls_gpu_last_error(void);

/* Replaces SparseCsrOperator's constructor (sparse_csr_operator.cpp:14-130):
 * validates the CSR arrays (int64 offsets and indices, FP64 values, device
 * memory), copies them, builds the transpose and the certified norm model.
 * The caller may free its arrays afterwards. */
int amfls_gpu_csr_operator_create(int rows, int cols, const int64_t* d_row_offsets,
                                  const int64_t* d_column_indices, const double* d_values,
                                  int64_t nonzeros, void* stream, amfls_gpu_operator** out);

/* Dense operator over caller-owned device memory (not copied; keep it alive):
 * column_major = 0 is the row-major layout of RowMajorDenseOperator
 * (row_major_dense_operator.cpp), 1 the column-major DenseOperator
 * (dense_operator.cpp). */
int amfls_gpu_dense_operator_create(int rows, int cols, const double* d_values, int column_major,
                                    void* stream, amfls_gpu_operator** out);

/* A matrix-free operator over caller callbacks, the C-ABI form of the
 * reference's custom MatrixOperator subclasses (matrix_operator.hpp:29-89).
 * apply computes Y (rows x s) = A X (cols x s), apply_transpose X = A^T Y,
 * on column-major device blocks, enqueuing their work on `stream` (the
 * result must be ready in stream order); they return 0 on success.
 * relative_block_product_cost may be NULL (the interface default s).
 * Without a validation model (has_validation_model = 0) no solve certifies
 * success, as in the reference (matrix_operator.hpp:17-20).  The solver
 * calls the callbacks from the calling thread and never inside a CUDA graph
 * capture.  The context and callbacks must outlive the operator. */
typedef struct {
    void* context;
    int (*apply)(void* context, const double* d_x, int block_cols, double* d_y, void* stream);
    int (*apply_transpose)(void* context, const double* d_y, int block_cols, double* d_x,
                           void* stream);
    double (*relative_block_product_cost)(void* context, int block_cols);
    int has_validation_model;
    amfls_gpu_validation_error_model validation_model;
} amfls_gpu_operator_callbacks;

int amfls_gpu_callback_operator_create(int rows, int cols,
                                       const amfls_gpu_operator_callbacks* callbacks, void* stream,
                                       amfls_gpu_operator** out);

int amfls_gpu_operator_destroy(amfls_gpu_operator* op);
int amfls_gpu_operator_rows(const amfls_gpu_operator* op);
int amfls_gpu_operator_cols(const amfls_gpu_operator* op);

/* MatrixOperator::apply / apply_transpose (matrix_operator.hpp:36-44):
 * column-major device blocks X (cols x block_cols), Y (rows x block_cols). */
int amfls_gpu_operator_apply(const amfls_gpu_operator* op, const double* d_x, int block_cols,
                             double* d_y, void* stream);
int amfls_gpu_operator_apply_transpose(const amfls_gpu_operator* op, const double* d_y,
                                       int block_cols, double* d_x, void* stream);

/* MatrixOperator::relative_block_product_cost (matrix_operator.hpp:50-55). */
double amfls_gpu_operator_relative_block_product_cost(const amfls_gpu_operator* op,
                                                      int block_cols);

/* MatrixOperator::validation_error_model (matrix_operator.hpp:57-60). */
int amfls_gpu_operator_validation_error_model(const amfls_gpu_operator* op,
                                              amfls_gpu_validation_error_model* out);

/* solve_amfls (amfls.hpp:22-25): d_b (rows) and d_solution (cols) are device
 * vectors; trace_float (capacity x 29) and trace_int (capacity x 4) are host
 * buffers (may be NULL when trace_capacity is 0). Synchronous on `stream`. */
int amfls_gpu_solve_amfls(const amfls_gpu_operator* op, const double* d_b,
                          const amfls_gpu_options* options, double* d_solution,
                          amfls_gpu_result* result, double* trace_float, int64_t* trace_int,
                          int trace_capacity, void* stream);

/* solve_fixed_rbgk (fixed_rbgk.hpp:22-25), same conventions. */
int amfls_gpu_solve_fixed_rbgk(const amfls_gpu_operator* op, const double* d_b,
                               const amfls_gpu_options* options, double* d_solution,
                               amfls_gpu_result* result, double* trace_float, int64_t* trace_int,
                               int trace_capacity, void* stream);

/* solve_lsqr (lsqr.hpp:14-17; lsqr.cpp:84-281) and solve_lsmr (lsmr.hpp;
 * lsmr.cpp:112-351): scalar LSQR / LSMR on the same operators, every
 * checkpoint certified by the same validation as AMFLS; result, trace and
 * error conventions as amfls_gpu_solve_amfls (iterations = depth = basis
 * rank = the last certified iteration, auxiliary width 0). */
int amfls_gpu_solve_lsqr(const amfls_gpu_operator* op, const double* d_b,
                         const amfls_gpu_baseline_options* options, double* d_solution,
                         amfls_gpu_result* result, double* trace_float, int64_t* trace_int,
                         int trace_capacity, void* stream);
int amfls_gpu_solve_lsmr(const amfls_gpu_operator* op, const double* d_b,
                         const amfls_gpu_baseline_options* options, double* d_solution,
                         amfls_gpu_result* result, double* trace_float, int64_t* trace_int,
                         int trace_capacity, void* stream);

/* Mixed-precision form (no counterpart in the reference, whose solver is
 * FP64 throughout).
 *
 * amfls_gpu_reduced_operator_create: the matrix of a CSR or dense operator
 * made by amfls_gpu_csr_operator_create / amfls_gpu_dense_operator_create,
 * with its values rounded once (to nearest) to FP32 (value_type 1) or BF16
 * (value_type 2).  Products round x to FP32 and accumulate in FP32; the
 * operator takes and returns FP64 blocks like any other.  A CSR reduced
 * operator shares the source's index arrays: destroy it before the source.
 * Its validation model describes the rounded matrix (norm bounds widened by
 * the rounding, rounding steps counted in FP64 units: one FP32 step = 2^29).
 */
#define AMFLS_GPU_VALUES_FP32 1
#define AMFLS_GPU_VALUES_BF16 2
int amfls_gpu_reduced_operator_create(const amfls_gpu_operator* source, int value_type,
                                      void* stream, amfls_gpu_operator** out);

/* amfls_gpu_solve_amfls_mixed: solve_amfls's problem on `op` (FP64) by
 * iterative refinement: each outer step runs AMFLS with lambda = 0 to
 * inner_tolerance on `reduced` (lambda = 0) or on [reduced; sqrt(lambda) I]
 * (lambda > 0) for the correction of the current x, then validates x with
 * the certified FP64 validation on `op`.  It stops when that certificate
 * meets options->tolerance (status 0), when it no longer contracts, or after
 * maximum_refinements steps.  It no longer contracts when it fails to halve
 * after an inner solve that reached inner_tolerance, or, for inner solves
 * cut by options->maximum_depth (restart cycles: pass a tiny
 * inner_tolerance and the cycle length as maximum_depth), when it fails to
 * fall below 0.99 of its best value two steps earlier.  When the steps on
 * `reduced` stop contracting and `reduced` is not `op`, the remaining steps
 * solve on `op` instead (precision schedule); `reduced` == `op` runs FP64
 * inner solves throughout.  options->reduced_basis applies to the inner
 * solves.  result->status / stop_reason and the metrics are those of the
 * last FP64 validation; depth and iterations add up the inner solves; one
 * trace row per outer step (column 0 the step, column 1 the levels so far,
 * column 2 1 when the step solved on `op`, column 3 the inner basis rank,
 * column 17 the step's relative energy error bound).  Same buffer
 * conventions as amfls_gpu_solve_amfls. */
int amfls_gpu_solve_amfls_mixed(const amfls_gpu_operator* op, const amfls_gpu_operator* reduced,
                                const double* d_b, const amfls_gpu_options* options,
                                double inner_tolerance, int maximum_refinements,
                                double* d_solution, amfls_gpu_result* result,
                                double* trace_float, int64_t* trace_int, int trace_capacity,
                                void* stream);

/* Learned width controller (no counterpart in the reference).
 *
 * A policy is an MLP (AMFLS_GPU_POLICY_INPUTS -> 32 -> 32 -> 1, tanh, FP64)
 * that scores the controller's two choices at each widening decision (the
 * reference's decision sites, amfls.cpp:319-359): the inputs are the
 * AMFLS_GPU_POLICY_FEATURES controller features followed by the action
 * (0 stay, 1 widen); the output predicts how fast the certificate falls
 * afterwards.  Parameters are AMFLS_GPU_POLICY_PARAMS doubles laid out
 * W1[32][12] b1[32] W2[32][32] b2[32] w3[32] b3.  Forward, gradient and
 * training (full-batch Adam on the mean squared error) run as CUDA kernels;
 * inputs, targets and parameters are host arrays; all are synchronous. */
#define AMFLS_GPU_POLICY_FEATURES 11
#define AMFLS_GPU_POLICY_INPUTS 12
#define AMFLS_GPU_POLICY_PARAMS 1505
/* one decision-log row: features[11], action, heuristic choice, rate
 * (decades of certificate per second until the next decision), valid */
#define AMFLS_GPU_DECISION_COLUMNS 15

typedef struct amfls_gpu_policy amfls_gpu_policy;

int amfls_gpu_policy_initial_params(uint64_t seed, double* params, int count);
int amfls_gpu_policy_create(const double* params, int count, amfls_gpu_policy** out);
int amfls_gpu_policy_destroy(amfls_gpu_policy* policy);
int amfls_gpu_policy_forward(const double* params, int count, const double* inputs, int n,
                             double* out, void* stream);
int amfls_gpu_policy_gradient(const double* params, int count, const double* inputs,
                              const double* targets, int n, double* grad, double* loss,
                              void* stream);
int amfls_gpu_policy_train(double* params, int count, const double* inputs, const double* targets,
                           int n, int epochs, double learning_rate, double* loss_first,
                           double* loss_last, void* stream);

/* solve_amfls with its width decisions controlled: with a policy the
 * policy's choice replaces the heuristic's (a non-finite score falls back to
 * the heuristic); with exploration in (0, 1] each decision is replaced by a
 * fair coin with that probability (seeded by exploration_seed).  Every
 * decision is logged to `decisions` (host, decision_capacity rows of
 * AMFLS_GPU_DECISION_COLUMNS; *decision_rows receives the count, rows beyond
 * the capacity are dropped).  policy NULL and exploration 0 give the
 * reference's controller.  Other conventions as amfls_gpu_solve_amfls. */
int amfls_gpu_solve_amfls_controlled(const amfls_gpu_operator* op, const double* d_b,
                                     const amfls_gpu_options* options,
                                     const amfls_gpu_policy* policy, double exploration,
                                     uint64_t exploration_seed, double* decisions,
                                     int decision_capacity, int* decision_rows,
                                     double* d_solution, amfls_gpu_result* result,
                                     double* trace_float, int64_t* trace_int, int trace_capacity,
                                     void* stream);

/* solve_amfls in schedule-replay mode (a test mode; the reference's
 * controller is amfls.cpp:57-661).  The controller's width decisions at its
 * decision sites (amfls.cpp:323-354, in order) take the candidate bits
 * replay[0 .. replay_count) instead of the bits its timing-driven cost gate
 * computes (amfls_internal.hpp:236-552); every other quantity of a decision
 * (increment, matched horizon) is computed as usual.  The bit is the only
 * timing-dependent part of a decision, so replaying the bits recorded from a
 * reference run reproduces that run's widening path on this GPU.  Sites
 * beyond the list keep their own bit and are counted in *replay_overrun;
 * replay_count < 0 replays nothing (the plain controller).  decisions
 * (capacity decision_capacity, may be NULL when 0) receives the bit taken at
 * every site and *decision_count the number of sites.  Other conventions as
 * amfls_gpu_solve_amfls. */
int amfls_gpu_solve_amfls_replay(const amfls_gpu_operator* op, const double* d_b,
                                 const amfls_gpu_options* options, const int* replay,
                                 int replay_count, int* decisions, int decision_capacity,
                                 int* decision_count, long long* replay_overrun,
                                 double* d_solution, amfls_gpu_result* result,
                                 double* trace_float, int64_t* trace_int, int trace_capacity,
                                 void* stream);

/* Measurement hook (no counterpart in the reference): times the two
 * width-one reorthogonalisation sweeps of a level (c = V^T r, then
 * r -> r - V c with its norm and DGKS test; krylov_workspace.cpp:152-165) on
 * a basis of n rows and k columns in the solver's own layout, filled with a
 * fixed pattern: `reps` launches of each after a warm-up, CUDA events on
 * `stream`.  seconds[0] and seconds[1] receive the mean seconds per launch of
 * the V^T r and the V c sweep.  Allocates 8 n k bytes for the duration of
 * the call; synchronous. */
int amfls_gpu_probe_reorthogonalization(int n, int k, int reps, void* stream, double* seconds);

/* The same for the reduced-basis sweeps (options.reduced_basis; no
 * counterpart in the reference): the first pass c = V~^T r~ on the FP32
 * (storage 1) or FP16 (storage 2) copy of the basis and r -> r - fl64(V~ c~).
 * seconds[0] / seconds[1] as above; *max_rel_error (may be NULL) receives
 * max_j |c_j - c64_j| / ||r||, the projection's deviation from the FP64
 * sweep on the same basis.  Allocates up to 12 n k bytes for the duration of
 * the call; synchronous. */
int amfls_gpu_probe_reorthogonalization_reduced(int n, int k, int reps, int storage,
                                                void* stream, double* seconds,
                                                double* max_rel_error);

/* The tiling of a CSR operator's single-column products (no counterpart in
 * the reference, whose products are scalar loops; sparse_csr_operator.cpp:
 * 203-269).  A side (A, or the stored transpose) is cut into warp tasks
 * either as chain groups or as row blocks; sides of at least 2^18 nonzeros
 * time both tilings when the operator is created and keep the faster one
 * when it wins by at least 10% over the size / row-length rule's choice; the
 * row-vector kernel (rows binned by length, 1-32 lanes per row, no shared
 * memory) is timed as a third candidate and replaces the tiles when it beats
 * the kept tiling by 5%.
 * chains[0], chains[1]: 0 when A's / the transpose's products use row
 * blocks, 1 chain groups, 2 the row-vector kernel; microseconds[0..3]: the
 * timed products of A with row blocks and with chain groups, then the
 * transpose's (0 where not timed).  An operator that is not a CSR operator
 * is AMFLS_GPU_INVALID_ARGUMENT. */
int amfls_gpu_csr_operator_schedule(const amfls_gpu_operator* op, int* chains,
                                    double* microseconds);

/* Batched AMFLS (no counterpart in the reference): `count` independent
 * problems, problem i = (ops[i], d_b[i], options[i]) with its solution in
 * d_solutions[i] (a distinct operator per problem: an operator's products
 * use scratch it owns), solved concurrently by `workers` host threads with one
 * CUDA stream each (streams created and destroyed inside the call),
 * largest problems (by nonzeros, or rows x cols) first.  results[i] as from
 * amfls_gpu_solve_amfls (trace rows counted, not copied); seconds[i] (may be
 * NULL) the wall time of problem i; *wall_seconds (may be NULL) the whole
 * batch.  Returns the first problem's error if any solve raised (the others
 * still run); synchronous. */
int amfls_gpu_solve_amfls_batch(int count, const amfls_gpu_operator* const* ops,
                                const double* const* d_b, const amfls_gpu_options* options,
                                double* const* d_solutions, amfls_gpu_result* results,
                                double* seconds, int workers, double* wall_seconds);

/* x = A^T y for a row-major dense A (rows x cols) without any device
 * allocation.  No counterpart in the reference: this is for callers that
 * cannot call cudaMalloc (code running during CUDA stream capture, real-time
 * loops that must not synchronise the device, hosts whose memory manager
 * owns all device memory).  The partial sums live in one fixed 8 MiB array
 * of device global memory (1,048,576 doubles) that every GPU loading the
 * library holds until exit; cols above that capacity are rejected with
 * AMFLS_GPU_LENGTH_ERROR.  The first call on each device looks the array's
 * device address up (cudaGetSymbolAddress) with that device current, so make
 * that first call before any stream capture.  The address is cached for the
 * life of the device's primary context: after cudaDeviceReset (or another
 * teardown of that context) do not call this entry point again in the
 * process.  All calls share the array:
 * calls whose kernels may overlap on the GPU (unordered streams) race; calls
 * ordered on one stream are safe.  Asynchronous on `stream`. */
int amfls_gpu_dense_apply_transpose_noalloc(int rows, int cols, const double* d_values,
                                            const double* d_y, double* d_x, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* AMFLS_GPU_H */
