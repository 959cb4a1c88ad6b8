// chf_internal.h -- handle layout, device buffers and kernel launchers.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/chflow.h"
#include "fft_dev.cuh"

namespace chf {

using cd = cplx<double>;
using cf = cplx<float>;

// Field slots of the resident state (the paraandcons.f90:28-38 arrays).
enum Field { F_V = 0, F_OY, F_U, F_W, F_OX, F_OZ, F_RV, F_RG, F_COUNT };
enum Mean { M_CL1N = 0, M_CL1NM1, M_CL3N, M_CL3NM1, M_AU0, M_W0, M_COUNT };

struct Dims {
  int nnx, nny, nnz;
  int N;    // Chebyshev degree (= nnz)
  int NZ;   // N + 1 coefficients / Gauss-Lobatto points
  int KX;   // streamwise complex modes kept = nnx/2
  int KY;   // spanwise complex modes = nny (slot NYQ unused)
  int NYQ;  // spanwise Nyquist slot = nny/2
  int PX;   // padded streamwise points = 3 nnx / 2
  int PY;   // padded spanwise points = 3 nny / 2
  int MZ;   // product-grid intervals in z (2 nnz in the reference)
  int MP;   // product-grid points = MZ + 1
  // Channels stacked in one set of buffers (an ensemble class of identical
  // grids, chf_batch.cu): KY = nch * nny spanwise slots, channel c in slots
  // c nny .. c nny + nny - 1, so a plane is [channel][ky][kx] and the z
  // passes, GEMMs and solves see nch times the modes; NYQ and the FFT passes
  // stay per channel.  chm = modes of one channel.  nch = 1: one channel.
  int nch;
  long chm;
  __host__ __device__ long modes() const { return (long)KX * KY; }
  __host__ __device__ size_t field_elems() const { return (size_t)NZ * KY * KX; }  // complex elements
};

// The Dims the x/y FFT passes see: one channel's spanwise modes, and the
// product-grid planes of every stacked channel as separate planes (a plane
// p of channel c is plane p nch + c).  The identity for one channel.
__host__ __device__ inline Dims fft_view(Dims d) {
  d.KY /= d.nch;
  d.MP *= d.nch;
  d.nch = 1;
  d.chm = (long)d.KX * d.KY;
  return d;
}

// Tensor-core GEMM plans (k_tcgemm.cu): K in chunks of at most TC_KC.
constexpr int TC_KC = 32;
constexpr int FX_PLANES = 4;     // digit planes per operand (the most a plan uses)
constexpr int FX_NT = 64;        // columns per B tile
struct FxPlan {
  int mvalid, mtiles, kpad, ntiles, nchunks;
  // digit format: 4 planes of 7-bit digits (levels 0..3, about 2^-28 of the
  // row and column maxima), or 3 planes of 8-bit digits (levels 0..2, about
  // 2^-24: for transforms whose output is FP32)
  int planes;
  long ncols;
  int kc[24];  // K <= 680 (the exactness bound) in chunks of TC_KC
  size_t a_chunk_off[24], b_chunk_off[24];
  size_t a_tile_bytes, b_tile_bytes;  // one 128-row A tile / one 64-column B tile
  __host__ __device__ size_t b_field_bytes() const { return (size_t)ntiles * b_tile_bytes; }
  __host__ __device__ size_t bexp_stride() const { return (size_t)ntiles * FX_NT; }
};

template <typename T>
struct Ptr8 {
  T* p[8];
};

// Even/odd split of the collocation operators (see k_solve.cu).
struct SolveLayout {
  int ne_v, no_v;  // even / odd unknowns of the v equation
  int ne_w, no_w;  // even / odd unknowns of the omega_y equation
  size_t stride;   // doubles per k^2 entry: ne_v^2 + no_v^2 + ne_w^2 + no_w^2
};

// Offsets of the four blocks (v even, v odd, omega even, omega odd) inside
// one k^2 entry of the inverses; each block column-major, X[c * n + r].
struct BlockOffsets {
  size_t ve, vo, we, wo;
};

__host__ __device__ inline BlockOffsets block_offsets(const SolveLayout& s) {
  BlockOffsets b;
  b.ve = 0;
  b.vo = b.ve + (size_t)s.ne_v * s.ne_v;
  b.we = b.vo + (size_t)s.no_v * s.no_v;
  b.wo = b.we + (size_t)s.ne_w * s.ne_w;
  return b;
}

// Launch shapes chosen by measurement (chf_tune.cu).  0 = the rule of the
// launcher (the largest shape that fits).
struct Tuning {
  int kxb = 0;      // streamwise modes per CTA of the shared-memory y transforms
  int xr = 0;       // (plane, y) rows per CTA of the shared-memory x transform
  int zl_c2v = 0;   // modes per CTA of the FP64 z transform to the product grid
  int zl_curl = 0;  // modes per CTA of the FP64 z transform + curl
  int inc_mch = 4;  // modes per CTA (work item) of the increment solve (2 or 4)
  int inc_cb = 4;   // matrix columns per load batch of the increment solve (2..4)
  int inc_rpt = 1;  // rows per thread of the increment solve (1 or 2; 2 with 2 or 3 columns)
  int inc_wide = 1; // one row per thread: every block row in one pass (1) or loop (0)
  // arithmetic of k_inc_recover (not searched by the autotuner): -1 the
  // handle's rule, 0 FP64, 1 double-float (2^-44 relative)
  int rec_form = -1;
  bool tuned = false;
  bool manual = false;  // a shape was set by chf_set_launch_shape
};

struct Handle {
  chf_config cfg;
  Tuning tune;
  Dims d;
  int device = 0;
  int num_sms = 1;  // multiprocessors of the device (persistent-kernel grids)
  cudaStream_t stream = nullptr;
  std::string err;
  bool uploaded = false;

  // resident state, FP64 (identical layout to the host arrays)
  cd* f[F_COUNT] = {};
  double* mean[M_COUNT] = {};  // each 2*NZ doubles, (2,0:nz)

  // wavenumbers
  double* iapha = nullptr;  // KX
  double* ibeta = nullptr;  // KY
  // Chebyshev collocation matrices (SCHEB), column-major NZ x NZ
  double *t0 = nullptr, *t2 = nullptr, *t4 = nullptr;
  // implicit operator inverses per distinct k^2 (even/odd blocks)
  SolveLayout sl{};
  int nk2 = 0;
  double* k2vals = nullptr;   // nk2
  double* xinv = nullptr;     // nk2 * sl.stride
  // mixed solve (k_solve_mixed.cu), per k^2: A^-1 (B - A) as (hi, lo)
  // floats, A^-1 as floats, and per row the exponent of sum |hi| over the row
  float2* incm = nullptr;
  float* incx = nullptr;
  signed char* incr_exp = nullptr;
  // k_inc_solve work items {group, first mode index}: runs of at most 4
  // modes (n_inc_items[1] of them), then runs of at most 2 (n_inc_items[0])
  int2* inc_items = nullptr;
  int n_inc_items[2] = {0, 0};
  bool rec_df_rule = false;  // k_inc_recover's double-float form (setup_solver_mixed)
  double* xmean = nullptr;    // inverse of the (0,0) operator, NZ x NZ column-major
  int* group_start = nullptr; // nk2 + 1 (modes grouped by k^2)
  int* group_modes = nullptr; // solved modes, sorted by k^2 index
  int nsolve = 0;
  // constant flow rate (chf_set_flow_rate): influence function, its bulk
  // velocity, device word {target, correction, bulk before, bulk after}
  double* phi = nullptr;
  double ubphi = 0.0;
  double* flow = nullptr;
  // stacked channels (d.nch > 1): per-group Reynolds number (group_re[g],
  // the (0,0) groups nk2 .. nk2 + nch - 1 last), per-channel phi [nch][NZ],
  // flow words [nch][4] and bulk velocities of phi (ubphi_dev[nch])
  double* group_re = nullptr;
  double* ubphi_dev = nullptr;

  // FFT plans and twiddles
  FftPlan py, px, pz2, pzm;   // PY, PX, 2N, 2MZ
  // PY, PX for FP64 lines when the nonlinear front is FP32 (the Lamb vector of
  // chf_pressure/chf_lamb on a mixed handle): the radix-8 rule and the launch
  // rules, never the FP32 tuning, so those results equal an FP64 handle's
  FftPlan py64, px64;
  // stage twiddle tables of the two-buffer x / y stages (fft_stage_twiddles),
  // PY / PX entries each: of py and px in the precision of the handle's
  // x / y lines (cf for a mixed front, cd for CHF_FP64), and of py64 and px64
  // in FP64 (mixed handles); rebuilt whenever a plan changes
  // (upload_stage_twiddles)
  void *stw_py = nullptr, *stw_px = nullptr;
  cd *stw_py64 = nullptr, *stw_px64 = nullptr;
  cd *tw_py = nullptr, *tw_px = nullptr, *tw_z2 = nullptr, *tw_zm = nullptr;
  cf *twf_py = nullptr, *twf_px = nullptr;

  // work buffers
  cd* wz = nullptr;   // 6 x [MP][KY][KX]  (values on the product grid)
  cd* wy = nullptr;   // 6 x [MP][PY][KX]  (after the spanwise transform)
  void* scratch = nullptr;  // reduction scratch (diagnostics)
  void* stats_buf = nullptr;  // chf_statistics: GL values of u, v, w + plane sums (first call)
  void* pres_buf = nullptr;   // chf_pressure: Lamb coefficients, right-hand sides, P (first call)
  // physical space (chf_phys.cu, first call): three field-sized FP64
  // buffers, plane maxima, and the unpadded x / y transform plans
  void* phys_buf = nullptr;
  FftPlan pxu{}, pyu{};       // nnx, nny
  cd *tw_pxu = nullptr, *tw_pyu = nullptr;
  size_t scratch_bytes = 0;

  // mixed-precision path (k_mixed.cu): FP32 transforms, tcgen05 GEMMs
  int* dev_status = nullptr;  // device error word (tensor-core pipeline timeouts)
  // chf_test_wait_timeout: the next exact-GEMM launch leaves its first stage
  // empty and bounds its waits at test_wait_ns
  int test_skip = 0;
  long test_wait_ns = 0;
  FxPlan tz1{}, tz2{}, tgl{};
  uint8_t *az1 = nullptr, *az2 = nullptr, *agl = nullptr;  // constant A images
  uint8_t* bimg = nullptr;    // per-step B images
  int *aexp1 = nullptr, *aexp2 = nullptr, *aexp3 = nullptr;  // row exponents of the A images
  int* bexp = nullptr;        // per-step column exponents of the fixed-point B images
  // row N of the Z2 and GL transforms (their GEMMs cover rows 0..N-1): the
  // rows' digit planes [4][kpad] and exponents
  float *z2_tail = nullptr, *gl_tail = nullptr;
  int z2_tail_exp = 0, gl_tail_exp = 0;
  size_t bimg_bytes = 0;
  cf* wz32 = nullptr;         // 6 x [MP][KY][KX]
  cf* wy32 = nullptr;         // 6 x [MP][PY][KX]
  double* lc64 = nullptr;     // 3 x [NZ][2 modes] Lamb-vector coefficients (exact z transform)

  // statistics
  int kernels_per_step = 0;
  cudaStream_t own_stream = nullptr;
  // mixed path: the (0,0)-mode solve runs on a side stream beside the other
  // modes' solve (fork / join events on the handle's stream)
  cudaStream_t side_stream = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // chf_step_host: copy streams in / out and the events that order them
  // against the handle's stream; after_inc, when set, is recorded right after
  // the mixed path's increment solve (v, omega_y final from there on)
  cudaStream_t copy_in = nullptr, copy_out = nullptr;
  cudaEvent_t ev_ready = nullptr, ev_inputs = nullptr, ev_hist_in = nullptr, ev_nonlinear = nullptr,
              ev_vg = nullptr, ev_done = nullptr;
  cudaEvent_t after_inc = nullptr;
  cudaEvent_t ev_field[6] = {};  // the six nonlinear inputs landed (u, v, w, omega_x, omega_y, omega_z)

  // chf_step replays a CUDA graph of two steps.  Each step exchanges the
  // history buffers by pointer (f[F_U] <-> f[F_RV], f[F_W] <-> f[F_RG]), so
  // a pair of steps restores the arrangement and one graph, keyed by the
  // arrangement it was captured in, serves every later pair.
  struct StepGraph {
    cd* f[F_COUNT];
    cudaGraphExec_t exec;
  };
  std::vector<StepGraph> graphs;
  bool graphs_off = false;  // capture failed once: launch directly from then on

  // per-kernel event timing (chf_profile_*)
  struct ProfRec {
    const char* name;
    int launches;
    double ms;
  };
  struct ProfPending {
    int kid;
    cudaEvent_t a, b;
  };
  bool profiling = false;
  std::vector<ProfRec> prof;
  std::vector<ProfPending> pending;
  std::vector<cudaEvent_t> event_pool;
};

// Kernel ids for profiling.
enum KernelId {
  K_ZC2V = 0, K_YINV, K_XPROD, K_YFWD, K_ZCURL, K_SOLVE, K_DIAG,
  K_SPLIT_Z1, K_GEMM_Z1, K_SPLIT_Z2, K_GEMM_Z2, K_CURL32, K_GEMM_GL, K_MEANFIX,
  K_INC_SOLVE, K_INC_RECOVER, K_SOLVE_MEAN, K_COUNT
};
extern const char* const kKernelNames[K_COUNT];

// Bracket one launch with events when profiling is on.
void prof_begin(Handle* h, int kid, cudaEvent_t* a);
void prof_end(Handle* h, int kid, cudaEvent_t a);

bool cuda_ok(Handle* h, cudaError_t e, const char* what);

// launchers (k_nonlinear.cu)
int launch_nonlinear_fp64(Handle* h);
int launch_lamb_fp64(Handle* h, cd* hc);
template <typename T>
int launch_xy(Handle* h, cplx<T>* wz, cplx<T>* wy, const cplx<T>* tw_py, const cplx<T>* tw_px);
// launchers (k_tcgemm.cu, k_mixed.cu)
// Wall-normal transforms as tcgen05 GEMMs (k_tcgemm.cu): operands as FX_PLANES planes of
// signed 7-bit integer digits below a per-row (A) / per-column (B) power of
// two, products of digits accumulated exactly per level i + j <= 3.
// 128-row A tiles, 64-column B tiles (two CTAs per SM fit in TMEM).
FxPlan make_fx_plan(int mvalid, int kvalid, long ncols, int planes = FX_PLANES);
std::vector<uint8_t> make_a_image_fx(const FxPlan& p, const std::vector<double>& a, int M, int K,
                                     std::vector<int>& row_exp);
template <typename OutT>
int launch_tc_gemm_fx(Handle* h, const FxPlan& p, const uint8_t* aimg, const int* aexp, const uint8_t* bimg,
                      const int* bexp, const Ptr8<OutT>& outs, int nfields, size_t ldc, int kid);
// One GEMM output row computed beside the split instead of by an extra row
// tile: the row's digit planes (device, plane-major, kpad each), its exponent,
// and per field the FP64 destination of the row.
struct FxTail {
  const float* adig = nullptr;
  int aexp = 0;
  Ptr8<double> out{};
};
std::vector<float> a_row_digits(const FxPlan& p, const std::vector<double>& a, int K, int row, int& row_exp);
template <typename InT>
int launch_tc_split_fx(Handle* h, const FxPlan& p, const Ptr8<const InT>& ins, int kvalid, uint8_t* bimg,
                       int* bexp, int nfields, int kid, const FxTail& tail = FxTail{});
int setup_mixed(Handle* h);
// field_ready (optional): six events, one per nonlinear input in the order
// u, v, w, omega_x, omega_y, omega_z; when given, each field's share of the
// first stages waits for its own event only (chf_step_host's upload)
int launch_nonlinear_mixed(Handle* h, const cudaEvent_t* field_ready = nullptr);
// precision of the handle's stages (chf_api.cu): the mixed nonlinear front
// (CHF_MIXED, CHF_MIXED_F64SOLVE) and the increment solve (CHF_MIXED only;
// CHF_FP64 and CHF_MIXED_F64SOLVE run the FP64 k_solve)
bool mixed_front(const Handle* h);
bool increment_solve(const Handle* h);
// getnonlinear / the solve of the handle's precision, on h->stream
int launch_nonlinear(Handle* h, const cudaEvent_t* field_ready);
int launch_solve(Handle* h);
// one time step (getnonlinear + solve) on h->stream (chf_api.cu)
int step_once(Handle* h);
// launchers (k_solve.cu)
int setup_solver(Handle* h);
int setup_solver_mixed(Handle* h);
// the work items of k_inc_solve from the handle's k^2 groups
int setup_inc_items(Handle* h);
// (re)writes the stage twiddle tables of h->py, h->px, h->py64, h->px64
// (allocated on the first call); synchronous, outside stream capture
int upload_stage_twiddles(Handle* h);
bool xy_register_path(const Dims& d);
int launch_yinv_fields(Handle* h, cf* wz, cf* wy, const cf* tw_py, int f0, int nf);
int launch_xprod_yfwd(Handle* h, cf* wz, cf* wy, const cf* tw_py, const cf* tw_px);
int launch_solve_fp64(Handle* h);
int launch_solve_mean(Handle* h, cudaStream_t st);  // the (0,0) mode alone, on st
int launch_solve_mixed(Handle* h);  // k_solve_mixed.cu
int launch_diagnostics(Handle* h, chf_diag* out);

// FFT plan helpers (host): radices 4, 2, 3, 5 for the in-place stages;
// the largest radices up to maxr for the two-buffer stages
FftPlan make_plan(int L);
FftPlan make_plan_pp(int L, int maxr);
// autotuner (chf_tune.cu): launch shapes the rules accept for a knob (0 kxb,
// 1 xr, 2 zl_c2v, 3 zl_curl; k_nonlinear.cu), and the process's cached
// choice for a new handle's key
std::vector<int> shape_candidates(const Handle* h, int knob);
void apply_cached_tuning(Handle* h);
// tw[k] = exp(-2 pi i k / L), k = 0..L-1 (host, libm)
std::vector<cd> twiddles(int L);
}  // namespace chf
