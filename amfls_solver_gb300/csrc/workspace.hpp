// Block Golub-Kahan workspace on the device.
//
// GB300 restatement of BlockGolubKahanWorkspace
// (src/algorithms/mathematics/krylov/krylov_workspace.hpp:93-189 and
// krylov_workspace.cpp:335-963).  Data layout in HBM:
//   V  right basis, n x k FP64, stored as panels of 32 columns; panel p is a
//      row-major n x 32 tile (row i of the panel = 256 contiguous bytes), so a
//      sweep over V reads contiguous 2 KB runs and a new column is one
//      strided write.  Panels are allocated on demand and never moved.
//   U  active left block, m x w column-major (only the unconsumed frontier,
//      as in the reference); P pending P*Omega, m x p.
//   T  projected operator: lower bidiagonal at width one, kept as the two
//      diagonals alpha_j = T(j, j), beta_{j+1} = T(j+1, j); g = U^T b.
// Width-one levels run entirely on the device (DevState decisions): one level
// is captured as the body of a CUDA graph WHILE node, so a whole checkpoint
// interval is a single graph launch.  Wider blocks use the host-synchronised
// block path.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <memory>
#include <vector>

#include "device_operator.hpp"
#include "vector_ops.hpp"
#include "workspace_state.hpp"

namespace amfls_gpu {


// Panels of 32 columns, each a row-major n x 32 tile, with a device table of
// their addresses.  T = double holds V; T = float its reduced-basis shadow.
template <typename T>
class PanelStoreT {
public:
    PanelStoreT(int n, int max_panels, cudaStream_t stream);
    ~PanelStoreT();
    void ensure_columns(int cols);  // allocate (zeroed) panels to hold `cols` columns
    T* column(int j) const { return host_[j / 32] + (j % 32); }  // stride 32
    T* const* device_table() const { return table_; }
    int panels() const { return static_cast<int>(host_.size()); }
    int n() const { return n_; }
    size_t bytes() const { return host_.size() * static_cast<size_t>(n_) * 32 * sizeof(T); }

private:
    int n_;
    cudaStream_t stream_;
    std::vector<T*> host_;
    T** table_ = nullptr;
    int table_cap_ = 0;
};
using PanelStore = PanelStoreT<double>;
using PanelStore32 = PanelStoreT<float>;
using PanelStore16 = PanelStoreT<__half>;

// Storage of the reduced-basis copy of V (options.reduced_basis).
enum ReducedStorage { kReducedOff = 0, kReducedFp32 = 1, kReducedFp16 = 2 };

class Workspace {
public:
    // reduced_basis (a ReducedStorage): width-one levels keep an FP32 or FP16
    // copy of V and run their first projection pass on it (see
    // enqueue_level_kernels).
    Workspace(const DeviceOperator& op, const double* d_b, double regularization,
              int maximum_basis_size, cudaStream_t stream, bool time_operators,
              bool use_graphs = true, int reduced_basis = kReducedOff);
    ~Workspace();
    Workspace(const Workspace&) = delete;
    Workspace& operator=(const Workspace&) = delete;

    // krylov_workspace.cpp:470-503; the auxiliary block (m x cols, device,
    // column-major) may be null when cols == 0.
    void initialize(const double* d_aux, int aux_cols);
    // krylov_workspace.cpp:505-587
    int append_left_seed(const double* d_seed, int cols);
    // Enqueue levels until `target_depth` or until the process cannot
    // advance; no host synchronisation at width one.
    void advance_to(int target_depth);
    // One level, synchronised (widening trials).
    bool advance_level();
    // Copy the device state back (a synchronisation point).
    void sync();

    int depth() const { return host_.depth; }
    int basis_rank() const { return host_.k; }
    int basis_limit() const { return basis_limit_; }
    int active_left_width() const { return host_.left_width; }
    bool can_advance() const {
        return initialized_ && host_.reliable && host_.left_width + host_.pending > 0 &&
               host_.k < basis_limit_;
    }
    double right_hand_side_norm() const { return b_norm_; }
    const StepAudit& last_step_audit() const { return host_.audit; }
    const DevState& state() const { return host_; }

    // Projected solve (krylov_workspace.cpp:833-909): writes the candidate
    // x = V y into d_x (n).  Returns false when the projected problem was
    // flagged as numerically rank deficient (see projected_flags()).
    void solve_projected(double* d_x);
    int projected_flags() const { return projected_flags_; }

    // accumulated device timings of search operator calls since the last call
    void take_operator_seconds(double& a_seconds, double& at_seconds);

    const DeviceOperator& op() const { return op_; }
    const double* b() const { return b_; }
    cudaStream_t stream() const { return stream_; }
    double* scratch_partials() const { return partials_; }
    unsigned* scratch_counter() const { return counter_; }

    // true once a level or seed wider than one column has been seen
    bool block_mode() const { return block_mode_; }
    // whether width-one levels project on a reduced copy of V
    bool reduced_basis() const { return reduced_basis_; }

private:
    // frees every device buffer, stream, graph and event the workspace holds
    // (the destructor, and a constructor that fails after allocating)
    void release() noexcept;
    void enqueue_level_kernels(cudaStream_t s, int pcap);
    void build_graph(int pcap);
    void invalidate_graph();
    void ensure_t_capacity(int cols);

    // ---- block (width > 1) levels, host-synchronised (block_level.cu) ----
    // Result of orthogonalize_and_factor (krylov_workspace.cpp:43-52, 82-310).
    struct Factor {
        int rank = 0;
        std::vector<double> coefficients;  // basis cols x block cols (when retained)
        std::vector<double> factor;        // rank x block cols
        double discarded = 0.0;
        double tracked = 0.0;
        double cutoff = 0.0;
        bool positive_below = false;
        bool nonfinite = false;
    };
    // basis: the panel-stored V (first `cols` columns) or a column-major
    // m x cols matrix
    struct Basis {
        bool panels;
        const double* mat;
        int cols;
    };
    Factor orthogonalize_and_factor(double* block, int cols, const Basis& basis, int max_rank,
                                    double scale, int tracked, bool retain, double* q_out);
    bool block_level();
    void enter_block_mode();
    void ensure_block_capacity(int width);
    void ensure_u_capacity(int cols);
    double device_norm(const double* x, long long count);
    double timed_apply(bool transpose, const double* in, int cols, double* out);
    void push_state();
    const double* block_projected_y(int* flags);  // y (k) of the record-based solve
    void upload(double* dst, const std::vector<double>& src);

    const DeviceOperator& op_;
    cudaStream_t stream_;
    int m_, n_;
    double reg_;
    int basis_limit_;
    bool initialized_ = false;
    bool time_ops_;
    bool use_graphs_;
    const double* b_;   // caller's device b (kept alive by the caller)
    double b_norm_ = 0.0;

    DevState host_{};
    DevState* dstate_ = nullptr;
    RedResult* red_ = nullptr;  // [4] reduction slots
    double* partials_ = nullptr;
    long long vc_partials_offset_ = 0;
    // basis sweeps (sweep_vt_kernel / sweep_vc_kernel): their grid, partial
    // sums, per-tile sums of squares and tickets (panels | tiles | done)
    int sweep_grid_ = 0;
    bool warp_sweeps_ = true;
    double* sweep_part_ = nullptr;
    double* sweep_sq_ = nullptr;
    unsigned* sweep_tickets_ = nullptr;
    long long sweep_panels_ = 0;
    unsigned* counter_ = nullptr;   // self-resetting tickets: misc + one per V panel

    std::unique_ptr<PanelStore> V_;
    // reduced-basis sweeps: FP32 or FP16 copy of V, r rounded to FP32, the FP32
    // coefficients, per-panel sums of c^2 and the tickets (panels | all)
    bool reduced_basis_ = false;
    int reduced_storage_ = kReducedOff;
    std::unique_ptr<PanelStore32> V32_;
    std::unique_ptr<PanelStore16> V16_;
    float* r32_ = nullptr;
    float* c32_ = nullptr;
    double* panel_sq_ = nullptr;
    unsigned* red_tickets_ = nullptr;
    double* red_part_ = nullptr;
    int red_grid_ = 0;
    double* U_ = nullptr;      // m x ucap
    int ucap_ = 0;
    double* P_ = nullptr;      // m x pcap (pending seed)
    int pcap_ = 0;
    double* R_ = nullptr;      // n residual
    double* vnew_ = nullptr;   // n
    double* Y_ = nullptr;      // m residual
    double* c1_ = nullptr;     // coefficients (k cap)
    double* c2_ = nullptr;
    int ccap_ = 0;
    // projected operator at width one
    double* alpha_ = nullptr;  // T(j,j)
    double* beta_ = nullptr;   // T(j+1,j)
    double* g_ = nullptr;      // g
    int tcap_ = 0;
    // incremental Givens QR of [T; sqrt(lambda) I]
    double* qr_ = nullptr;     // rho, theta, phi (3 x tcap) + y (tcap)
    double* qr_state_ = nullptr;  // [c, s, rhobar, phibar, processed]
    int projected_flags_ = 0;
    // one width-one level captured as the body of a device-side WHILE loop
    cudaStream_t capture_stream_ = nullptr;
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t graph_exec_ = nullptr;
    int graph_pcap_ = 0;  // V panels the captured sweep grids cover
    long long body_kernels_ = 0;       // kernels in the captured level body
    long long counted_body_runs_ = 0;  // body runs already added to launch_count()
    long long graph_launches_ = 0;
    unsigned long long seen_a_ns_ = 0, seen_at_ns_ = 0;

    // block mode state (host side; device buffers below)
    bool block_mode_ = false;
    int pending_requested_ = 0;
    int pending_retained_ = 0;
    std::vector<double> coupling_;  // frontier coupling, left_width x prev_right_width
    // level records of T: meta (r, aw, nlw, value offset, state offset) and
    // values G | N | g (see block.hpp)
    std::vector<int> rec_meta_;
    std::vector<double> rec_vals_;
    long long rec_state_size_ = 0;
    int rec_last_r_ = 0;
    int rec_width_ = 1;
    int rec_solved_ = 0;  // levels folded into the projected-solve carry
    int* d_meta_ = nullptr;
    long long d_meta_cap_ = 0;
    double* d_vals_ = nullptr;
    long long d_vals_cap_ = 0;
    long long d_vals_uploaded_ = 0;
    int d_meta_uploaded_ = 0;
    double* d_pstate_ = nullptr;
    long long d_pstate_cap_ = 0;
    double* d_carry_ = nullptr;
    long long d_carry_cap_ = 0;
    double* d_pwork_ = nullptr;
    long long d_pwork_cap_ = 0;
    double* d_y_ = nullptr;
    long long d_y_cap_ = 0;
    // block scratch
    int bcap_ = 0;             // block width the residual buffers hold
    double* BR_ = nullptr;     // n x bcap right residual
    double* BL_ = nullptr;     // m x bcap left residual / seed
    double* BQ_ = nullptr;     // n x bcap new right block
    double* BT_ = nullptr;     // max(m, n) x bcap block before re-orthogonalisation
    double* U2_ = nullptr;     // m x ucap next left block
    double* small_ = nullptr;  // factorisation scratch (width^2 sized)
    long long small_cap_ = 0;
    double* coefs_ = nullptr;  // two passes of basis^T block coefficients
    long long coefs_cap_ = 0;
    double* bpart_ = nullptr;  // partial sums of the tall-skinny products
    long long bpart_cap_ = 0;
    double* tsqr_ = nullptr;
    long long tsqr_cap_ = 0;
    int* dflags_ = nullptr;    // [0] nonfinite coefficients, [1] Cholesky, [2] projected
    NormResult* dnorm_ = nullptr;
    cudaEvent_t ev_[2] = {nullptr, nullptr};
};

// Times the width-one reorthogonalisation sweeps (c = V^T r and the
// r -> r - V c pass with its norm and DGKS test, krylov_workspace.cpp:152-165)
// exactly as a level launches them, on a basis of n rows and k columns in the
// panel layout filled with a fixed pattern: `reps` launches of each, CUDA
// events on `stream`; seconds[0] / seconds[1] receive the mean per launch.
void probe_reorthogonalization(int n, int k, int reps, cudaStream_t stream, double seconds[2]);
// The same for the reduced-basis sweeps (an FP32 or FP16 copy of V, a
// ReducedStorage; FP32 products, FP64 subtraction): seconds[0] / seconds[1]
// the V~^T r and r - V~ c passes;
// max_rel_error[0] receives max |c - c_fp64| / ||r|| over the columns (the
// projection's error against the FP64 sweep on the same basis).
void probe_reorthogonalization_reduced(int n, int k, int reps, int storage,
                                       cudaStream_t stream, double seconds[2],
                                       double* max_rel_error);

}  // namespace amfls_gpu
