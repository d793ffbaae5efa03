// Internal declarations of the dachshund-gb300 CUDA library.
//
// Layout in HBM (one operator):
//   * pixel coordinates as three FP64 SoA arrays x[], y[], z[] in a spatially
//     sorted order (3-D Morton order of the points scaled by the correlation
//     lengths), padded to a multiple of TILE with copies of the last point;
//   * per-pixel operator coefficients in the same order: wl (left scale),
//     wr (right scale), e (diagonal), b (right-hand side), pdiag (Jacobi);
//     padding rows carry zeros, so padded vector entries stay exactly zero;
//   * perm[] (sorted -> caller index) and the per-tile bounding boxes;
//   * the culled tile-pair list in CSR form (row tile -> column tiles).
// All vectors that iterate (x, r, d, q, s) live in sorted order; the caller's
// order is restored only at the API boundary.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "ds_gb300.h"

namespace ds {

struct OpF32;   // ds_f32.h
struct MapF32;  // ds_f32.h
struct SkewerPC;  // ds_learned.h
struct SkewerGrid;  // ds_skewer.h
struct MapColumns;  // ds_skewer.h
struct OpF32Deleter { void operator()(OpF32* p) const; };
struct MapF32Deleter { void operator()(MapF32* p) const; };
struct SkewerPCDeleter { void operator()(SkewerPC* p) const; };
struct SkewerGridDeleter { void operator()(SkewerGrid* p) const; };
struct MapColumnsDeleter { void operator()(MapColumns* p) const; };

constexpr int TILE = 128;        // points per tile (rows per CTA in the FP64 kernels)
constexpr int SUBTILE = 32;      // points per sub-tile (one warp's rows; culled per warp)
constexpr int TABLE_N = DS_TABLE_N;

struct Error {
  int code;
  std::string msg;
};

#define DS_CUDA(call)                                                        \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess)                                                   \
      throw ::ds::Error{e_ == cudaErrorMemoryAllocation ? DS_ERR_OOM         \
                                                        : DS_ERR_CUDA,       \
                        std::string(#call) + ": " + cudaGetErrorString(e_)}; \
  } while (0)

// Every kernel launch of the library is followed by DS_CHECK_LAUNCH(), which
// also counts it (process-wide).
long long& launch_counter();
#define DS_CHECK_LAUNCH()          \
  do {                             \
    ++::ds::launch_counter();      \
    DS_CUDA(cudaGetLastError());   \
  } while (0)

inline void require(bool ok, const char* msg) {
  if (!ok) throw Error{DS_ERR_ARG, msg};
}

// Stream on which device buffers are allocated and freed in stream order
// (cudaMallocAsync / cudaFreeAsync from the device's memory pool, which the
// context keeps cached): the calling context's stream while a library call
// runs (set by guarded()), otherwise none (plain cudaMalloc / cudaFree, which
// synchronise the device).  A buffer is freed on the stream it was allocated
// on, after the work queued there; objects are destroyed before their
// context.
inline thread_local cudaStream_t g_alloc_stream = nullptr;

// Streams of the live contexts (registered at ds_context_create, removed
// before ds_context_destroy destroys the stream).  A buffer allocated in
// stream order is freed in stream order while its stream exists, else with
// cudaFree (which waits for the device), so an object destroyed after its
// context (as a garbage collector may order it) never names a dead stream.
bool stream_alive(cudaStream_t s);
void stream_register(cudaStream_t s, bool alive);

// Device buffer (owning).
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaStream_t s = nullptr;  // allocation stream (stream-ordered) when async
  bool async = false;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), n(o.n), s(o.s), async(o.async) {
    o.p = nullptr;
    o.n = 0;
    o.async = false;
  }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      n = o.n;
      s = o.s;
      async = o.async;
      o.p = nullptr;
      o.n = 0;
      o.async = false;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(size_t count) {
    if (count == n && p) return;
    release();
    if (count == 0) return;
    s = g_alloc_stream;
    async = s != nullptr;
    if (async)
      DS_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&p), count * sizeof(T), s));
    else
      DS_CUDA(cudaMalloc(&p, count * sizeof(T)));
    n = count;
  }
  void release() {
    if (p) {
      if (async && stream_alive(s))
        cudaFreeAsync(p, s);
      else
        cudaFree(p);
    }
    p = nullptr;
    n = 0;
    async = false;
  }
  size_t bytes() const { return n * sizeof(T); }
};

// Pinned host buffer.
template <class T>
struct HostBuf {
  T* p = nullptr;
  size_t n = 0;
  HostBuf() = default;
  HostBuf(const HostBuf&) = delete;
  HostBuf& operator=(const HostBuf&) = delete;
  ~HostBuf() { if (p) cudaFreeHost(p); }
  void alloc(size_t count) {
    if (count <= n && p) return;
    if (p) cudaFreeHost(p);
    p = nullptr;
    n = 0;
    DS_CUDA(cudaMallocHost(&p, count * sizeof(T)));
    n = count;
  }
};

// Kernel constants shared by every pair kernel.
struct KernelConsts {
  double var_s;
  double c_perp;     // 1 / (2 l_perp^2)
  double c_para;     // 1 / (2 l_para^2)
  double dx_inv;     // table index scale, 199/8
  double exact_cut;  // exponent cutoff of the exact kernel
  double cull_arg;   // tile-pair culling threshold on c_perp dperp^2 + c_para dz^2
  int eval;          // DS_EVAL_TABLE / DS_EVAL_EXACT
};

KernelConsts make_consts(const ds_kernel_params& kp);
void host_table(double* table, double* dx_inv);

// A spatially sorted, tiled point set on the device.
struct PointSet {
  int n = 0;
  int n_pad = 0;
  int n_tiles = 0;
  DevBuf<double> x, y, z;  // sorted + padded
  DevBuf<int> perm;        // sorted position -> caller index (-1 on padding)
  DevBuf<double> box;      // 6 per tile: lo x, y, z, hi x, y, z
  DevBuf<double> sbox;     // 6 per SUBTILE-point sub-tile, same layout
  // FP32 copies rounded outward (lo down, hi up), each containing its FP64
  // box: the pair search's culling tests
  DevBuf<float> box32, sbox32;
};

// Builds a PointSet from n records of `stride` doubles (x, y, z first) that
// are already in device memory.  sx, sy, sz scale the coordinates for the
// spatial key only (the stored coordinates are unscaled).
// order: ORDER_MORTON cuts the Morton-sorted sequence into tiles (cheap; good
// for regular grids); ORDER_KD refines it into a balanced k-d partition with
// exactly TILE points per tile (compact boxes for scattered pixels).
enum PointOrder { ORDER_MORTON = 0, ORDER_KD = 1 };
void build_point_set(PointSet& ps, const double* d_rec, int n, int stride,
                     double sx, double sy, double sz, cudaStream_t st,
                     int order = ORDER_KD);
// Bounding box of n records of `stride` doubles (x, y, z first) in device
// memory; DS_ERR_ARG for a non-finite coordinate (synchronises st).
void point_bbox(const double* d_rec, int n, int stride, double lo[3], double hi[3],
                cudaStream_t st);

// Culled tile-pair list (CSR over row tiles).
struct PairList {
  int n_rows = 0;
  long long n_pairs = 0;
  DevBuf<int> row_ptr;  // n_rows + 1
  DevBuf<int> cols;     // n_pairs
  // per pair: bit (4 k + w) set when row sub-tile k interacts with column
  // sub-tile w (the same box test at sub-tile granularity)
  DevBuf<unsigned short> mask;
  DevBuf<int> row_order;  // row tiles by decreasing pair count (launch order)
  // Work items of the FP32 kernels (build_slice_items): per tile pair, one
  // per column sub-tile w with some interacting row sub-tile, in tile-pair
  // then w order; entry = column tile << 6 | w << 4 | row sub-tiles (bit k).
  DevBuf<int> item_ptr;         // n_rows + 1
  DevBuf<unsigned int> items;
};

void build_pair_list(PairList& pl, const PointSet& rows, const PointSet& cols,
                     const KernelConsts& kc, cudaStream_t st);
void build_slice_items(PairList& pl, cudaStream_t st);

// ---- pair kernels (FP64) -------------------------------------------------
// Column weight u_j and epilogue selection.
enum PairEpi {
  EPI_PRODUCT = 0,   // out_i = wl_i acc + e_i v_i      (u_j = wr_j v_j)
  EPI_RESIDUAL = 1,  // out_i = b_i - (wl_i acc + e_i v_i)
  EPI_MAP = 2,       // out[perm_i] = acc               (u_j = v_j)
  EPI_NOISE = 3      // out[perm_i] = sum S^2 u_j       (u_j = 1 / N_j)
};

struct PairArgs {
  // geometry
  const double* rx; const double* ry; const double* rz;
  const double* cx; const double* cy; const double* cz;
  const int* row_ptr; const int* cols;
  int n_row_tiles;
  const unsigned short* mask;  // sub-tile interaction mask per tile pair
  const int* row_order;        // blockIdx -> row tile (heaviest first), or null
  // coefficients (sorted order)
  const double* wl; const double* wr; const double* e; const double* b;
  const double* v;      // the vector being multiplied (column side)
  const double* vrow;   // the same vector on the row side (diagonal term)
  double* out;
  const int* row_perm;  // EPI_MAP / EPI_NOISE scatter
  // fused dot product: partial[tile] = sum_i dotv_i out_i (if dot_partial)
  const double* dotv;
  double* dot_partial;
  // early exit when *skip_flag != 0
  const int* skip_flag;
  // last-block reduction of dot_partial -> pcg alpha
  struct PcgState* pcg;
  unsigned int* counter;
  const double* table;  // TABLE_N knots
  // profiling: total evaluated pairs of this launch, added on the device by
  // launches that ran (not by those that exited on skip_flag)
  long long n_tile_pairs;
  unsigned long long* prof_pairs;
  struct Profiler* prof;
};

// Per-context event timing of pair-kernel launches (ds_context_set_profiling).
// Kinds: 0 = FP64-accurate pair kernels (products, residuals), 1 = FP32 pair
// kernels (products), 2 = map products (FP64 or FP32), 3 = dense matvecs
// (their "pairs" are matrix entries read).
struct Profiler {
  struct Pending {
    cudaEvent_t start, stop;
    int kind;
  };
  bool enabled = false;
  std::vector<cudaEvent_t> free_events;
  std::vector<Pending> pending;
  static constexpr int KINDS = 4;
  long long launches[KINDS] = {0, 0, 0, 0};
  double ms[KINDS] = {0.0, 0.0, 0.0, 0.0};
  unsigned long long* d_pairs = nullptr;  // device counters of evaluated pairs, per kind
  cudaEvent_t get_event();
  void begin(cudaStream_t st, cudaEvent_t* ev);
  void end(cudaStream_t st, cudaEvent_t start, int kind);
  void collect();  // waits for pending events and folds them into the totals
  ~Profiler();
};

void launch_pair_f64(const KernelConsts& kc, int epi, const PairArgs& a,
                     cudaStream_t st);

// ---- PCG -----------------------------------------------------------------
struct PcgState {
  double delta;       // r . s (current)
  double delta_old;
  double alpha;
  double beta;
  double dq;
  double norm_r;
  double norm_b;
  double tol_norm_b;
  int iter;           // completed iterations
  int max_iter;
  int done;
  int converged;
  unsigned int counter[4];
};

}  // namespace ds

// Opaque handles of the C ABI.
struct ds_context {
  int device = 0;
  int num_sms = 0;  // streaming multiprocessors of the device (persistent grids)
  long long wait_limit = 0;  // bound of tensor-core mbarrier waits (0: default)
  cudaStream_t stream = nullptr;
  std::string last_error;
  ds::Profiler prof;
};

struct ds_operator {
  ds_context* ctx = nullptr;
  int form = 0;
  int n = 0;
  ds::KernelConsts kc{};
  ds::PointSet pix;
  ds::PairList pairs;
  ds::DevBuf<double> table;
  ds::DevBuf<double> wl, wr, e, b;  // sorted, padded operator coefficients
  ds::DevBuf<double> pdiag;         // Jacobi diagonal (1 on padding)
  ds::DevBuf<int> inv;              // caller index -> sorted position
  ds::DevBuf<double> io_a, io_b;    // caller-order device staging
  double norm_b = 0.0;
  // PCG work space (sorted, padded)
  ds::DevBuf<double> x, r, d, q, s, tmp, tmp2;
  ds::DevBuf<double> partial;      // per-block partial sums
  ds::DevBuf<double> partial2;
  ds::DevBuf<ds::PcgState> state;
  ds::DevBuf<double> hist, dhist;  // residual norms and deltas per iteration
  ds::HostBuf<double> h_io;        // pinned staging
  ds::HostBuf<int> h_flag;
  unsigned long long serial = 0;   // identity for caches keyed on operators
  std::unique_ptr<ds::OpF32, ds::OpF32Deleter> f32;  // mixed-precision data (lazy)
  ds::DevBuf<double> dense;  // dense A (n_pad x n_pad, sorted order) when enabled
  bool use_dense = false;
  // dense matvec: arithmetic (ds_dense_arith; float pairs need every nonzero
  // |A_ij| in [2^-100, 2^100], recorded at build time with the sign), the
  // float-pair copy of the vector, per-column-block row partials, per-row-block
  // dot partials and arrival counters (n_pad / 64 + 1, zero between launches)
  int dense_arith = 0;
  bool dense_ff_ok = false;
  bool dense_signed = false;
  ds::DevBuf<float2> dense_vff;
  ds::DevBuf<double> dense_part, dense_dot;
  ds::DevBuf<unsigned int> dense_cnt;
  bool pairs_built = false;  // `pairs` (ensure_op_pairs)
  int inner_variant = 0;     // inner matvec of the mixed form (InnerVariant)
  int iter_form = 0;         // DS_ITER_AUTO / DS_ITER_GRAPH
  // skewer-band preconditioner of the mixed form (null: Jacobi)
  std::unique_ptr<ds::SkewerPC, ds::SkewerPCDeleter> pc;
  // structured operator for skewers on a shared z grid (null: pair kernels)
  std::unique_ptr<ds::SkewerGrid, ds::SkewerGridDeleter> sgrid;
};

struct ds_map {
  ds_context* ctx = nullptr;
  int n = 0;                  // map points
  ds::DevBuf<double> raw;     // the points as given (x, y, z each), caller order
  ds::PointSet pts;           // tiled copy, built on first use (ensure_map_points)
  bool pts_built = false;
  // pair list cache for the last operator used
  unsigned long long op_serial = 0;
  ds::KernelConsts kc{};
  ds::PairList pairs;
  ds::DevBuf<double> out_dev;  // caller-order map staging
  std::unique_ptr<ds::MapF32, ds::MapF32Deleter> f32;  // FP32 map data (lazy)
  // map points declared a column grid (null: none), for the structured map
  std::unique_ptr<ds::MapColumns, ds::MapColumnsDeleter> cols;
};
