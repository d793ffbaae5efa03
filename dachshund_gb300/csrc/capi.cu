// The C ABI (include/ds_gb300.h): argument checks, host <-> device staging,
// object lifetimes and the mapping of internal errors to status codes.
#include <atomic>
#include <mutex>
#include <unordered_set>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

#include "ds_batch.h"
#include "ds_device.cuh"
#include "ds_f32.h"
#include "ds_ops.h"
#include "ds_skewer.h"

namespace ds {

static std::mutex& streams_mutex() {
  static std::mutex m;
  return m;
}
static std::unordered_set<cudaStream_t>& live_streams() {
  static std::unordered_set<cudaStream_t> s;
  return s;
}

bool stream_alive(cudaStream_t s) {
  std::lock_guard<std::mutex> lock(streams_mutex());
  return live_streams().count(s) != 0;
}

void stream_register(cudaStream_t s, bool alive) {
  std::lock_guard<std::mutex> lock(streams_mutex());
  if (alive)
    live_streams().insert(s);
  else
    live_streams().erase(s);
}

void ensure_map_points(ds_map* map) {
  if (map->pts_built) return;
  build_point_set(map->pts, map->raw.p, map->n, 3, 1.0, 1.0, 1.0, map->ctx->stream,
                  ORDER_MORTON);
  map->pts_built = true;
}

}  // namespace ds

using namespace ds;

namespace {

std::atomic<unsigned long long> g_serial{1};

constexpr int VB = 256;
inline int grid_for(long long n) {
  return (int)std::max<long long>(1, std::min<long long>(4096, (n + VB - 1) / VB));
}

// Sorted operator coefficients from the caller's records (lib/wf_vector.cc
// 140-147 for SN, 283-292 for W):
//   SN: wl = wr = 1, e = N,  b = d,  Jacobi diagonal var_s + N
//   W:  wl = wr = w, e = 1,  b = wd, Jacobi diagonal w^2 var_s + 1
__global__ void k_op_coeffs(int n_pad, int form, double var_s, const int* __restrict__ perm,
                            const double* __restrict__ rec, double* __restrict__ wl,
                            double* __restrict__ wr, double* __restrict__ e,
                            double* __restrict__ b, double* __restrict__ pdiag,
                            int* __restrict__ inv) {
  for (int i = blockIdx.x * VB + threadIdx.x; i < n_pad; i += gridDim.x * VB) {
    const int p = perm[i];
    if (p < 0) {
      wl[i] = wr[i] = e[i] = b[i] = 0.0;
      pdiag[i] = 1.0;
      continue;
    }
    inv[p] = i;
    const double f = rec[(size_t)p * 5 + 3];
    const double rhs = rec[(size_t)p * 5 + 4];
    if (form == DS_FORM_SN) {
      wl[i] = wr[i] = 1.0;
      e[i] = f;
      pdiag[i] = __dadd_rn(var_s, f);
    } else {
      wl[i] = wr[i] = f;
      e[i] = 1.0;
      pdiag[i] = __dadd_rn(__dmul_rn(__dmul_rn(f, f), var_s), 1.0);
    }
    b[i] = rhs;
  }
}

// x = M^-1 b in caller order.
__global__ void k_precond(int n, const int* __restrict__ inv, const double* __restrict__ pdiag,
                          const double* __restrict__ src, double* __restrict__ dst) {
  for (int i = blockIdx.x * VB + threadIdx.x; i < n; i += gridDim.x * VB)
    dst[i] = src[i] / pdiag[inv[i]];
}

// WFVector{SN,W}::A(i, j, exact), lib/wf_vector.cc:16-40 and 157-183.
__global__ void k_entries(KernelConsts kc, int form, int m, const int* __restrict__ ii,
                          const int* __restrict__ jj, const int* __restrict__ inv,
                          const double* __restrict__ x, const double* __restrict__ y,
                          const double* __restrict__ z, const double* __restrict__ wl,
                          const double* __restrict__ e, const double* __restrict__ table,
                          double* __restrict__ out) {
  __shared__ double tf[TABLE_N];
  for (int k = threadIdx.x; k < TABLE_N; k += blockDim.x) tf[k] = table[k];
  __syncthreads();
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    const int i = ii[k], j = jj[k];
    const int si = inv[i], sj = inv[j];
    const double dx = x[si] - x[sj], dy = y[si] - y[sj], dz = z[si] - z[sj];
    const double S = kc.eval == DS_EVAL_TABLE ? s_table_f64(dx, dy, dz, kc, tf)
                                              : kc.var_s * exp(-(kc.c_perp * (dx * dx + dy * dy) +
                                                                 kc.c_para * (dz * dz)));
    const double delta = (i == j) ? 1.0 : 0.0;
    out[k] = form == DS_FORM_SN ? __dadd_rn(S, __dmul_rn(e[si], delta))
                                : __dadd_rn(__dmul_rn(__dmul_rn(wl[si], S), wl[sj]), delta);
  }
}

__global__ void k_signal_covar(KernelConsts kc, int n, const double* __restrict__ perp2,
                               const double* __restrict__ para2, const double* __restrict__ table,
                               double* __restrict__ out) {
  __shared__ double tf[TABLE_N];
  for (int k = threadIdx.x; k < TABLE_N; k += blockDim.x) tf[k] = table[k];
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double S;
    if (kc.eval == DS_EVAL_TABLE) {
      // signal_covar, lib/signal_covar.h:67-77, from precomputed squares.
      const double g = __dadd_rn(__dmul_rn(kc.c_perp, perp2[i]), __dmul_rn(kc.c_para, para2[i]));
      const double xx = __dmul_rn(g, kc.dx_inv);
      int ix = __double2int_rz(xx);
      if (!(xx < (double)(TABLE_N - 1))) {
        S = 0.0;
      } else {
        ix = min(max(ix, 0), TABLE_N - 2);
        const double gp = __dadd_rn(__dmul_rn(tf[ix], __dsub_rn((double)(ix + 1), xx)),
                                    __dmul_rn(tf[ix + 1], __dsub_rn(xx, (double)ix)));
        S = __dmul_rn(kc.var_s, gp);
      }
    } else {
      // signal_covar_exact, lib/signal_covar.h:79-86 (no cutoff here).
      S = kc.var_s * exp(-(kc.c_perp * perp2[i] + kc.c_para * para2[i]));
    }
    out[i] = S;
  }
}

// u_j = 1 / N_j in sorted order (sigma_m_noise_dom weights).
__global__ void k_gather_recip_field(int n_pad, const int* __restrict__ perm,
                                     const double* __restrict__ rec, int stride, int field,
                                     double* __restrict__ dst) {
  for (int i = blockIdx.x * VB + threadIdx.x; i < n_pad; i += gridDim.x * VB) {
    const int p = perm[i];
    dst[i] = p >= 0 ? 1.0 / rec[(size_t)p * stride + field] : 0.0;
  }
}

void upload(const double* h, size_t n, DevBuf<double>& d, cudaStream_t st) {
  d.alloc(n);
  DS_CUDA(cudaMemcpyAsync(d.p, h, n * sizeof(double), cudaMemcpyHostToDevice, st));
}

ds_kernel_params checked_kp(const ds_kernel_params* kp) {
  require(kp != nullptr, "kernel params are null");
  return *kp;
}

void load_table(DevBuf<double>& table, const ds_kernel_params& kp, cudaStream_t st) {
  double h[TABLE_N];
  if (kp.table)
    std::memcpy(h, kp.table, sizeof(h));
  else
    host_table(h, nullptr);
  table.alloc(TABLE_N);
  DS_CUDA(cudaMemcpyAsync(table.p, h, sizeof(h), cudaMemcpyHostToDevice, st));
  DS_CUDA(cudaStreamSynchronize(st));  // h is on this stack frame
}

void op_product_dev(ds_operator* op, int epi, const double* a_dev, double* b_dev) {
  cudaStream_t st = op->ctx->stream;
  op->tmp.alloc(op->pix.n_pad);
  op->tmp2.alloc(op->pix.n_pad);
  gather_sorted(op->pix, a_dev, op->tmp.p, st);
  op_apply_sorted(op, epi, op->tmp.p, op->tmp2.p, st);
  scatter_sorted(op->pix, op->tmp2.p, nullptr, b_dev, st);
}

int op_host_call(ds_operator* op, int epi, const double* in, double* out) {
  if (!op) return DS_ERR_ARG;
  return guarded(op->ctx, [&] {
    require(in && out, "null vector");
    cudaStream_t st = op->ctx->stream;
    upload(in, op->n, op->io_a, st);
    op->io_b.alloc(op->n);
    op_product_dev(op, epi, op->io_a.p, op->io_b.p);
    DS_CUDA(cudaMemcpyAsync(out, op->io_b.p, op->n * sizeof(double), cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaStreamSynchronize(st));
  });
}

void ensure_map_pairs(ds_map* map, ds_operator* op) {
  ensure_map_points(map);
  if (map->op_serial == op->serial) return;
  build_pair_list(map->pairs, map->pts, op->pix, op->kc, map->ctx->stream);
  map->op_serial = op->serial;
  map->kc = op->kc;
}

void map_product_dev(ds_map* map, ds_operator* op, const double* x_dev, double* m_dev) {
  cudaStream_t st = map->ctx->stream;
  ensure_map_pairs(map, op);
  op->tmp.alloc(op->pix.n_pad);
  gather_sorted(op->pix, x_dev, op->tmp.p, st);
  PairArgs a{};
  a.rx = map->pts.x.p;
  a.ry = map->pts.y.p;
  a.rz = map->pts.z.p;
  a.cx = op->pix.x.p;
  a.cy = op->pix.y.p;
  a.cz = op->pix.z.p;
  a.row_ptr = map->pairs.row_ptr.p;
  a.cols = map->pairs.cols.p;
  a.mask = map->pairs.mask.p;
  a.row_order = map->pairs.row_order.p;
  a.n_row_tiles = map->pts.n_tiles;
  a.v = op->tmp.p;
  a.out = m_dev;
  a.row_perm = map->pts.perm.p;
  a.table = op->table.p;
  a.n_tile_pairs = map->pairs.n_pairs;
  a.prof = &map->ctx->prof;
  launch_pair_f64(op->kc, EPI_MAP, a, st);
}

}  // namespace

extern "C" {

const char* ds_status_string(int status) {
  switch (status) {
    case DS_OK: return "ok";
    case DS_ERR_ARG: return "invalid argument";
    case DS_ERR_CUDA: return "CUDA error";
    case DS_ERR_NOT_CONVERGED: return "PCG reached max iteration before stop condition";
    case DS_ERR_NORM_B: return "requested PCG solve where |b| <= 0";
    case DS_ERR_OOM: return "out of memory";
    case DS_ERR_NO_DEVICE: return "no usable CUDA device";
    case DS_ERR_STATE: return "object in error state";
    case DS_ERR_TIMEOUT: return "a bounded wait in a tensor-core kernel timed out";
    default: return "unknown status";
  }
}

void ds_table_init(double* table, double* dx_inv) { host_table(table, dx_inv); }

int ds_context_create(int device, ds_context** out) {
  if (!out) return DS_ERR_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) return DS_ERR_NO_DEVICE;
  if (device < 0 || device >= count) return DS_ERR_ARG;
  auto ctx = std::make_unique<ds_context>();
  ctx->device = device;
  const int rc = guarded(nullptr, [&] {
    DS_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    DS_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major < 10) throw Error{DS_ERR_NO_DEVICE, "device is not a Blackwell-class GPU"};
    ctx->num_sms = prop.multiProcessorCount;
    DS_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    stream_register(ctx->stream, true);
    // stream-ordered device buffers come from the default pool; keep what is
    // freed cached for the next allocations
    cudaMemPool_t pool;
    DS_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
    uint64_t keep = ~0ull;
    DS_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
  });
  if (rc != DS_OK) return rc;
  *out = ctx.release();
  return DS_OK;
}

void ds_context_destroy(ds_context* ctx) {
  if (!ctx) return;
  if (ctx->stream) {
    cudaStreamSynchronize(ctx->stream);
    stream_register(ctx->stream, false);
    cudaStreamDestroy(ctx->stream);
  }
  delete ctx;
}

void* ds_context_stream(ds_context* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int ds_context_synchronize(ds_context* ctx) {
  if (!ctx) return DS_ERR_ARG;
  return guarded(ctx, [&] { DS_CUDA(cudaStreamSynchronize(ctx->stream)); });
}

const char* ds_context_last_error(ds_context* ctx) {
  return ctx ? ctx->last_error.c_str() : "null context";
}

int ds_context_set_profiling(ds_context* ctx, int enable) {
  if (!ctx) return DS_ERR_ARG;
  return guarded(ctx, [&] {
    Profiler& p = ctx->prof;
    p.collect();
    if (enable) {
      const size_t bytes = Profiler::KINDS * sizeof(unsigned long long);
      if (!p.d_pairs) DS_CUDA(cudaMalloc(&p.d_pairs, bytes));
      DS_CUDA(cudaMemsetAsync(p.d_pairs, 0, bytes, ctx->stream));
      DS_CUDA(cudaStreamSynchronize(ctx->stream));
      for (int k = 0; k < Profiler::KINDS; ++k) {
        p.launches[k] = 0;
        p.ms[k] = 0.0;
      }
    }
    p.enabled = enable != 0;
  });
}

int ds_context_set_wait_limit(ds_context* ctx, long long cycles) {
  if (!ctx || cycles < 0) return DS_ERR_ARG;
  ctx->wait_limit = cycles;
  return DS_OK;
}

int ds_context_get_profile(ds_context* ctx, ds_profile* out) {
  if (!ctx || !out) return DS_ERR_ARG;
  return guarded(ctx, [&] {
    Profiler& p = ctx->prof;
    p.collect();
    unsigned long long pairs[Profiler::KINDS] = {0, 0, 0, 0};
    if (p.d_pairs) {
      DS_CUDA(cudaStreamSynchronize(ctx->stream));
      DS_CUDA(cudaMemcpy(pairs, p.d_pairs, sizeof(pairs), cudaMemcpyDeviceToHost));
    }
    out->f64_launches = p.launches[0];
    out->f64_ms = p.ms[0];
    out->f64_evaluated = (double)pairs[0];
    out->f32_launches = p.launches[1];
    out->f32_ms = p.ms[1];
    out->f32_evaluated = (double)pairs[1];
    out->map_launches = p.launches[2];
    out->map_ms = p.ms[2];
    out->map_evaluated = (double)pairs[2];
    out->dense_launches = p.launches[3];
    out->dense_ms = p.ms[3];
    out->dense_entries = (double)pairs[3];
    out->pair_launches = p.launches[0] + p.launches[1] + p.launches[2];
    out->pair_ms = p.ms[0] + p.ms[1] + p.ms[2];
    out->pair_evaluated = (double)pairs[0] + (double)pairs[1] + (double)pairs[2];
    out->kernel_launches = launch_counter();
  });
}

int ds_signal_covar(const ds_kernel_params* kp, int n, const double* perp2, const double* para2,
                    double* out) {
  return guarded(nullptr, [&] {
    const ds_kernel_params k = checked_kp(kp);
    require(n >= 0 && (n == 0 || (perp2 && para2 && out)), "bad arrays");
    if (n == 0) return;
    const KernelConsts kc = make_consts(k);
    cudaStream_t st = 0;
    DevBuf<double> table, dp, dq, dout;
    load_table(table, k, st);
    upload(perp2, n, dp, st);
    upload(para2, n, dq, st);
    dout.alloc(n);
    k_signal_covar<<<grid_for(n), VB, 0, st>>>(kc, n, dp.p, dq.p, table.p, dout.p);
    DS_CHECK_LAUNCH();
    DS_CUDA(cudaMemcpyAsync(out, dout.p, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaStreamSynchronize(st));
  });
}

int ds_operator_create(ds_context* ctx, int form, int n, const double* records,
                       const ds_kernel_params* kp, ds_operator** out) {
  if (!ctx || !out) return DS_ERR_ARG;
  *out = nullptr;
  auto op = std::make_unique<ds_operator>();
  const int rc = guarded(ctx, [&] {
    require(form == DS_FORM_SN || form == DS_FORM_W, "form must be DS_FORM_SN or DS_FORM_W");
    require(n > 0, "n must be > 0");
    require(records != nullptr, "records are null");
    const ds_kernel_params k = checked_kp(kp);
    DS_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    op->ctx = ctx;
    op->form = form;
    op->n = n;
    op->kc = make_consts(k);
    op->serial = g_serial++;
    load_table(op->table, k, st);
    DevBuf<double> rec;
    upload(records, (size_t)n * 5, rec, st);
    build_point_set(op->pix, rec.p, n, 5, std::sqrt(op->kc.c_perp), std::sqrt(op->kc.c_perp),
                    std::sqrt(op->kc.c_para), st);
    const int np = op->pix.n_pad;
    op->wl.alloc(np);
    op->wr.alloc(np);
    op->e.alloc(np);
    op->b.alloc(np);
    op->pdiag.alloc(np);
    op->inv.alloc(n);
    k_op_coeffs<<<grid_for(np), VB, 0, st>>>(np, form, op->kc.var_s, op->pix.perm.p, rec.p,
                                             op->wl.p, op->wr.p, op->e.p, op->b.p, op->pdiag.p,
                                             op->inv.p);
    DS_CHECK_LAUNCH();
    // the tile-pair list is built on the first pair-kernel call
    // (ensure_op_pairs): the structured operator needs none.
    // norm_b on the host in record order, as lib/wf_vector.cc:105-112, while
    // the device sorts and tiles the records.
    double sb2 = 0.0;
    for (int i = 0; i < n; ++i) sb2 += records[(size_t)i * 5 + 4] * records[(size_t)i * 5 + 4];
    op->norm_b = std::sqrt(sb2);
    DS_CUDA(cudaStreamSynchronize(st));
  });
  if (rc != DS_OK) return rc;
  *out = op.release();
  return DS_OK;
}

void ds_operator_destroy(ds_operator* op) {
  // cudaFree (in the buffer destructors) waits for work using the memory, so
  // the context (which may already be gone) is not touched here.
  delete op;
}

int ds_operator_get_info(ds_operator* op, ds_operator_info* info) {
  if (!op || !info) return DS_ERR_ARG;
  return guarded(op->ctx, [&] {
    ensure_op_pairs(op);
    info->n = op->n;
    info->n_pad = op->pix.n_pad;
    info->tile = TILE;
    info->n_tiles = op->pix.n_tiles;
    info->n_tile_pairs = op->pairs.n_pairs;
    info->evaluated_pairs = op->pairs.n_pairs * (long long)TILE * TILE;
  });
}

int ds_A_product(ds_operator* op, const double* a, double* b) {
  return op_host_call(op, EPI_PRODUCT, a, b);
}

int ds_A_residual(ds_operator* op, const double* x, double* r) {
  return op_host_call(op, EPI_RESIDUAL, x, r);
}

int ds_A_product_dev(ds_operator* op, const double* a, double* b) {
  if (!op) return DS_ERR_ARG;
  return guarded(op->ctx, [&] {
    require(a && b, "null vector");
    op_product_dev(op, EPI_PRODUCT, a, b);
  });
}

int ds_A_residual_dev(ds_operator* op, const double* x, double* r) {
  if (!op) return DS_ERR_ARG;
  return guarded(op->ctx, [&] {
    require(x && r, "null vector");
    op_product_dev(op, EPI_RESIDUAL, x, r);
  });
}

int ds_preconditioner_solve(ds_operator* op, const double* b, double* x) {
  if (!op) return DS_ERR_ARG;
  return guarded(op->ctx, [&] {
    require(b && x, "null vector");
    cudaStream_t st = op->ctx->stream;
    upload(b, op->n, op->io_a, st);
    op->io_b.alloc(op->n);
    k_precond<<<grid_for(op->n), VB, 0, st>>>(op->n, op->inv.p, op->pdiag.p, op->io_a.p,
                                               op->io_b.p);
    DS_CHECK_LAUNCH();
    DS_CUDA(cudaMemcpyAsync(x, op->io_b.p, op->n * sizeof(double), cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaStreamSynchronize(st));
  });
}

int ds_norm_b(ds_operator* op, double* norm_b) {
  if (!op || !norm_b) return DS_ERR_ARG;
  *norm_b = op->norm_b;
  return DS_OK;
}

int ds_A_entries(ds_operator* op, int eval, int m, const int* ii, const int* jj, double* out) {
  if (!op) return DS_ERR_ARG;
  return guarded(op->ctx, [&] {
    require(m >= 0 && (m == 0 || (ii && jj && out)), "bad arrays");
    require(eval == -1 || eval == DS_EVAL_TABLE || eval == DS_EVAL_EXACT, "bad eval");
    for (int k = 0; k < m; ++k)
      require(ii[k] >= 0 && ii[k] < op->n && jj[k] >= 0 && jj[k] < op->n, "index out of range");
    if (m == 0) return;
    cudaStream_t st = op->ctx->stream;
    KernelConsts kc = op->kc;
    if (eval >= 0) kc.eval = eval;
    DevBuf<int> di, dj;
    di.alloc(m);
    dj.alloc(m);
    DS_CUDA(cudaMemcpyAsync(di.p, ii, m * sizeof(int), cudaMemcpyHostToDevice, st));
    DS_CUDA(cudaMemcpyAsync(dj.p, jj, m * sizeof(int), cudaMemcpyHostToDevice, st));
    DevBuf<double> dout;
    dout.alloc(m);
    k_entries<<<grid_for(m), VB, 0, st>>>(kc, op->form, m, di.p, dj.p, op->inv.p, op->pix.x.p,
                                           op->pix.y.p, op->pix.z.p, op->wl.p, op->e.p,
                                           op->table.p, dout.p);
    DS_CHECK_LAUNCH();
    DS_CUDA(cudaMemcpyAsync(out, dout.p, m * sizeof(double), cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaStreamSynchronize(st));
  });
}

}  // extern "C"

// Shared frame of the solvers: initial guess in (host or device, caller
// order), solve in sorted order, W-form scaling x *= w, solution out.
template <class Solve>
static int solve_common(ds_operator* op, double* x, bool host, ds_pcg_result* res,
                        Solve&& solve) {
  if (!op || !x) return DS_ERR_ARG;
  int status = DS_OK;
  const int rc = guarded(op->ctx, [&] {
    cudaStream_t st = op->ctx->stream;
    ensure_pcg_workspace(op);
    double* xin = x;
    if (host) {
      upload(x, op->n, op->io_a, st);
      xin = op->io_a.p;
    }
    gather_sorted(op->pix, xin, op->x.p, st);
    ds_pcg_result r{};
    if (!(op->norm_b > 0.0)) {
      // lib/pcg.h:79-86: early return; the W form still scales x by w.
      puts("[WARNING] Requested PCG solve where |b| <= 0.0. Returning early.\n");
      r.norm_b = op->norm_b;
      status = DS_ERR_NORM_B;
    } else {
      solve(r);
      status = r.success ? DS_OK : DS_ERR_NOT_CONVERGED;
    }
    scatter_sorted(op->pix, op->x.p, op->form == DS_FORM_W ? op->wl.p : nullptr, xin, st);
    if (host) {
      DS_CUDA(cudaMemcpyAsync(x, xin, op->n * sizeof(double), cudaMemcpyDeviceToHost, st));
      DS_CUDA(cudaStreamSynchronize(st));
    }
    if (res) *res = r;
  });
  return rc != DS_OK ? rc : status;
}

extern "C" {

int ds_solve_pcg(ds_operator* op, const ds_pcg_params* pp, double* x, ds_pcg_result* res,
                 double* residual_norms) {
  if (!pp) return DS_ERR_ARG;
  return solve_common(op, x, true, res,
                      [&](ds_pcg_result& r) { run_pcg(op, *pp, r, residual_norms); });
}

int ds_solve_pcg_dev(ds_operator* op, const ds_pcg_params* pp, double* x, ds_pcg_result* res,
                     double* residual_norms) {
  if (!pp) return DS_ERR_ARG;
  return solve_common(op, x, false, res,
                      [&](ds_pcg_result& r) { run_pcg(op, *pp, r, residual_norms); });
}

int ds_A_residual_ff(ds_operator* op, const double* x, double* r) {
  if (!op) return DS_ERR_ARG;
  return guarded(op->ctx, [&] {
    require(x && r, "null vector");
    require(ff_usable(op->kc), "float-float residual needs DS_EVAL_EXACT and a cutoff <= 60");
    cudaStream_t st = op->ctx->stream;
    ensure_op_f32(op, op->f32 ? op->f32->inner_cut : DS_DEFAULT_INNER_CUTOFF);
    upload(x, op->n, op->io_a, st);
    op->io_b.alloc(op->n);
    op->tmp.alloc(op->pix.n_pad);
    op->tmp2.alloc(op->pix.n_pad);
    gather_sorted(op->pix, op->io_a.p, op->tmp.p, st);
    PairArgs a = op_pair_args(op, op->tmp.p, op->tmp2.p);
    launch_pair_ff_resid(op->kc, a, op->f32->ffd.view, st);
    scatter_sorted(op->pix, op->tmp2.p, nullptr, op->io_b.p, st);
    DS_CUDA(cudaMemcpyAsync(r, op->io_b.p, op->n * sizeof(double), cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaStreamSynchronize(st));
  });
}

int ds_solve_mixed(ds_operator* op, const ds_mixed_params* mp, double* x, ds_pcg_result* res,
                   double* residual_norms) {
  if (!mp) return DS_ERR_ARG;
  return solve_common(op, x, true, res,
                      [&](ds_pcg_result& r) { run_mixed(op, *mp, r, residual_norms); });
}

int ds_solve_mixed_dev(ds_operator* op, const ds_mixed_params* mp, double* x,
                       ds_pcg_result* res, double* residual_norms) {
  if (!mp) return DS_ERR_ARG;
  return solve_common(op, x, false, res,
                      [&](ds_pcg_result& r) { run_mixed(op, *mp, r, residual_norms); });
}

int ds_map_create(ds_context* ctx, int n_map, const double* map_points, ds_map** out) {
  if (!ctx || !out) return DS_ERR_ARG;
  *out = nullptr;
  auto map = std::make_unique<ds_map>();
  const int rc = guarded(ctx, [&] {
    require(n_map > 0 && map_points, "bad map points");
    cudaStream_t st = ctx->stream;
    map->ctx = ctx;
    map->n = n_map;
    // the points as given; the tiled copy is built by the first call that
    // needs it (a column-grid map against a skewer grid never does)
    upload(map_points, (size_t)n_map * 3, map->raw, st);
    double lo[3], hi[3];
    point_bbox(map->raw.p, n_map, 3, lo, hi, st);  // checks the coordinates
  });
  if (rc != DS_OK) return rc;
  *out = map.release();
  return DS_OK;
}

void ds_map_destroy(ds_map* map) { delete map; }

int ds_map_product_dev(ds_map* map, ds_operator* op, const double* x, double* m) {
  if (!map || !op) return DS_ERR_ARG;
  return guarded(map->ctx, [&] {
    require(x && m, "null vector");
    require(map->ctx == op->ctx, "map and operator belong to different contexts");
    map_product_dev(map, op, x, m);
  });
}

int ds_map_product(ds_map* map, ds_operator* op, const double* x, double* m) {
  if (!map || !op) return DS_ERR_ARG;
  return guarded(map->ctx, [&] {
    require(x && m, "null vector");
    require(map->ctx == op->ctx, "map and operator belong to different contexts");
    cudaStream_t st = map->ctx->stream;
    upload(x, op->n, op->io_a, st);
    map->out_dev.alloc(map->n);
    map_product_dev(map, op, op->io_a.p, map->out_dev.p);
    DS_CUDA(cudaMemcpyAsync(m, map->out_dev.p, map->n * sizeof(double),
                            cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaStreamSynchronize(st));
  });
}

int ds_map_product_f32_dev(ds_map* map, ds_operator* op, double cutoff, const double* x,
                           double* m) {
  if (!map || !op) return DS_ERR_ARG;
  return guarded(map->ctx, [&] {
    require(x && m, "null vector");
    require(map->ctx == op->ctx, "map and operator belong to different contexts");
    map_product_f32_dev(map, op, x, m, cutoff > 0.0 ? cutoff : 30.0);
  });
}

int ds_map_product_f32(ds_map* map, ds_operator* op, double cutoff, const double* x, double* m) {
  if (!map || !op) return DS_ERR_ARG;
  return guarded(map->ctx, [&] {
    require(x && m, "null vector");
    require(map->ctx == op->ctx, "map and operator belong to different contexts");
    cudaStream_t st = map->ctx->stream;
    upload(x, op->n, op->io_a, st);
    map->out_dev.alloc(map->n);
    map_product_f32_dev(map, op, op->io_a.p, map->out_dev.p, cutoff > 0.0 ? cutoff : 30.0);
    DS_CUDA(cudaMemcpyAsync(m, map->out_dev.p, map->n * sizeof(double),
                            cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaStreamSynchronize(st));
  });
}

int ds_smp_product(ds_context* ctx, int n_pix, const double* pixel_points, int n_map,
                   const double* map_points, const ds_kernel_params* kp, const double* x,
                   double* m) {
  if (!ctx) return DS_ERR_ARG;
  return guarded(ctx, [&] {
    require(n_pix > 0 && n_map > 0 && pixel_points && map_points && x && m, "bad arguments");
    const ds_kernel_params k = checked_kp(kp);
    const KernelConsts kc = make_consts(k);
    cudaStream_t st = ctx->stream;
    DevBuf<double> table, dpix, dmap, dx, xs, dm;
    load_table(table, k, st);
    upload(pixel_points, (size_t)n_pix * 3, dpix, st);
    upload(map_points, (size_t)n_map * 3, dmap, st);
    upload(x, n_pix, dx, st);
    PointSet pix, mp;
    build_point_set(pix, dpix.p, n_pix, 3, std::sqrt(kc.c_perp), std::sqrt(kc.c_perp),
                    std::sqrt(kc.c_para), st);
    build_point_set(mp, dmap.p, n_map, 3, 1.0, 1.0, 1.0, st, ORDER_MORTON);
    PairList pl;
    build_pair_list(pl, mp, pix, kc, st);
    xs.alloc(pix.n_pad);
    gather_sorted(pix, dx.p, xs.p, st);
    dm.alloc(n_map);
    PairArgs a{};
    a.rx = mp.x.p; a.ry = mp.y.p; a.rz = mp.z.p;
    a.cx = pix.x.p; a.cy = pix.y.p; a.cz = pix.z.p;
    a.row_ptr = pl.row_ptr.p;
    a.cols = pl.cols.p;
    a.mask = pl.mask.p;
    a.row_order = pl.row_order.p;
    a.n_row_tiles = mp.n_tiles;
    a.v = xs.p;
    a.out = dm.p;
    a.row_perm = mp.perm.p;
    a.table = table.p;
    a.n_tile_pairs = pl.n_pairs;
    a.prof = &ctx->prof;
    launch_pair_f64(kc, EPI_MAP, a, st);
    DS_CUDA(cudaMemcpyAsync(m, dm.p, n_map * sizeof(double), cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaStreamSynchronize(st));
  });
}

int ds_sigma_m_noise_dom(ds_context* ctx, int n_pix, const double* npixels, int n_map,
                         const double* map_points, const ds_kernel_params* kp, double* sigma_m) {
  if (!ctx) return DS_ERR_ARG;
  return guarded(ctx, [&] {
    require(n_pix > 0 && n_map > 0 && npixels && map_points && sigma_m, "bad arguments");
    const ds_kernel_params k = checked_kp(kp);
    const KernelConsts kc = make_consts(k);
    cudaStream_t st = ctx->stream;
    DevBuf<double> table, drec, dmap, u, dm;
    load_table(table, k, st);
    upload(npixels, (size_t)n_pix * 5, drec, st);
    upload(map_points, (size_t)n_map * 3, dmap, st);
    PointSet pix, mp;
    build_point_set(pix, drec.p, n_pix, 5, std::sqrt(kc.c_perp), std::sqrt(kc.c_perp),
                    std::sqrt(kc.c_para), st);
    build_point_set(mp, dmap.p, n_map, 3, 1.0, 1.0, 1.0, st, ORDER_MORTON);
    PairList pl;
    build_pair_list(pl, mp, pix, kc, st);
    u.alloc(pix.n_pad);
    k_gather_recip_field<<<grid_for(pix.n_pad), VB, 0, st>>>(pix.n_pad, pix.perm.p, drec.p, 5, 3,
                                                             u.p);
    DS_CHECK_LAUNCH();
    dm.alloc(n_map);
    PairArgs a{};
    a.rx = mp.x.p; a.ry = mp.y.p; a.rz = mp.z.p;
    a.cx = pix.x.p; a.cy = pix.y.p; a.cz = pix.z.p;
    a.row_ptr = pl.row_ptr.p;
    a.cols = pl.cols.p;
    a.mask = pl.mask.p;
    a.row_order = pl.row_order.p;
    a.n_row_tiles = mp.n_tiles;
    a.v = u.p;
    a.out = dm.p;
    a.row_perm = mp.perm.p;
    a.table = table.p;
    a.n_tile_pairs = pl.n_pairs;
    a.prof = &ctx->prof;
    launch_pair_f64(kc, EPI_NOISE, a, st);
    DS_CUDA(cudaMemcpyAsync(sigma_m, dm.p, n_map * sizeof(double), cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaStreamSynchronize(st));
  });
}

}  // extern "C"

extern "C" {

int ds_operator_set_dense(ds_operator* op, int enable) {
  if (!op) return DS_ERR_ARG;
  return guarded(op->ctx, [&] {
    if (enable) {
      if (!op->dense.p) op_build_dense(op);
      op->use_dense = true;
    } else {
      op->use_dense = false;
      op_free_dense(op);
    }
  });
}

int ds_operator_set_dense_arith(ds_operator* op, int arith) {
  if (!op) return DS_ERR_ARG;
  return guarded(op->ctx, [&] {
    require(arith >= DS_DENSE_AUTO && arith <= DS_DENSE_FP64, "bad dense arithmetic");
    op->dense_arith = arith;
  });
}

int ds_operator_get_dense_arith(ds_operator* op, int* arith) {
  if (!op || !arith) return DS_ERR_ARG;
  return guarded(op->ctx, [&] {
    require(op->dense.p != nullptr, "the dense operator is not built (ds_operator_set_dense)");
    *arith = dense_arith_in_use(op);
  });
}

int ds_operator_set_inner_matvec(ds_operator* op, int variant) {
  if (!op) return DS_ERR_ARG;
  return guarded(op->ctx, [&] {
    require(variant >= DS_INNER_AUTO && variant <= DS_INNER_STRUCTURED,
            "bad inner-matvec variant");
    op->inner_variant = variant;
  });
}

int ds_operator_set_iteration_form(ds_operator* op, int form) {
  if (!op) return DS_ERR_ARG;
  return guarded(op->ctx, [&] {
    require(form == DS_ITER_AUTO || form == DS_ITER_GRAPH, "bad iteration form");
    op->iter_form = form;
  });
}

int ds_operator_get_persistent_profile(ds_operator* op, double* out, int n, int reset,
                                       int* written) {
  if (!op || !out || n < 0) return DS_ERR_ARG;
  return guarded(op->ctx, [&] {
    const int m = persistent_profile(op, out, n, reset != 0);
    if (written) *written = m;
  });
}

int ds_solve_cf(ds_context* ctx, int form, int n, const double* records,
                const ds_kernel_params* kp, double* x) {
  if (!ctx) return DS_ERR_ARG;
  return guarded(ctx, [&] {
    require(form == DS_FORM_SN || form == DS_FORM_W, "form must be DS_FORM_SN or DS_FORM_W");
    require(n > 0 && records && x, "bad arguments");
    const ds_kernel_params k = checked_kp(kp);
    const KernelConsts kc = make_consts(k);
    cudaStream_t st = ctx->stream;
    DevBuf<double> table, rec, dx;
    load_table(table, k, st);
    upload(records, (size_t)n * 5, rec, st);
    dx.alloc(n);
    solve_cf_dev(ctx, form, n, rec.p, kc, table.p, dx.p);
    DS_CUDA(cudaMemcpyAsync(x, dx.p, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaStreamSynchronize(st));
  });
}

namespace {

// Right-hand sides b[k * R + r] = S(pixel k, map point r) (exact kernel, as
// the per-point path builds its column), zero for padding columns r >= m.
__global__ void k_mc_rhs(int n, int R, int m, const double* __restrict__ rec,
                         const double* __restrict__ mp, KernelConsts kc,
                         double* __restrict__ b) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)n * R) return;
  const int k = (int)(idx / R), r = (int)(idx % R);
  double v = 0.0;
  if (r < m) {
    const double dx = mp[3 * r] - rec[5 * (size_t)k], dy = mp[3 * r + 1] - rec[5 * (size_t)k + 1];
    const double dz = mp[3 * r + 2] - rec[5 * (size_t)k + 2];
    v = kc.var_s * exp(-(kc.c_perp * (dx * dx + dy * dy) + kc.c_para * dz * dz));
  }
  b[idx] = v;
}

// sig[r] = sum_k b[k R + r] x[k R + r] (one CTA per column, fixed order).
__global__ void k_mc_dot(int n, int R, const double* __restrict__ b, const double* __restrict__ x,
                         double* __restrict__ sig) {
  __shared__ double red[8];
  const int r = blockIdx.x;
  double s = 0.0;
  for (int k = threadIdx.x; k < n; k += blockDim.x)
    s = fma(b[(size_t)k * R + r], x[(size_t)k * R + r], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    sig[r] = t;
  }
}

// MapCovarDiag with the exact kernel: groups of MC_RHS map points are the
// right-hand sides of one batched mixed-precision SN-form solve over the
// pixels (ds_batch_*), so each kernel value of a pixel pair serves the whole
// group (and the tensor-core S-tile x RHS product applies); the per-point
// FP64 solves of the table kernel stay as the reference's path.
constexpr int MC_RHS = 64;

void map_covar_diag_batched(ds_context* ctx, int n_pix, const double* npixels, int n_map,
                            const double* map_points, const ds_kernel_params& kp,
                            const ds_pcg_params& pp, double* sigma_m, int* iters,
                            int* success) {
  cudaStream_t st = ctx->stream;
  ds_batch* batch = nullptr;
  const int sizes[1] = {n_pix};
  int rc = ds_batch_create(ctx, DS_FORM_SN, 1, sizes, npixels, &kp, MC_RHS, 0.0, &batch);
  if (rc != DS_OK) throw Error{rc, ctx->last_error};
  std::unique_ptr<ds_batch, void (*)(ds_batch*)> guard(batch, ds_batch_destroy);
  const KernelConsts kc = make_consts(kp);
  DevBuf<double> rec, mp, b, x, sig;
  upload(npixels, (size_t)n_pix * 5, rec, st);
  mp.alloc(3 * MC_RHS);
  b.alloc((size_t)n_pix * MC_RHS);
  x.alloc((size_t)n_pix * MC_RHS);
  sig.alloc(MC_RHS);
  std::vector<double> hp(3 * MC_RHS), hs(MC_RHS);
  std::vector<int> hit(MC_RHS), hconv(MC_RHS);
  const ds_mixed_params mpar{pp.max_iter, pp.tol, 0.0, 0.0, 0};
  for (int g = 0; g < n_map; g += MC_RHS) {
    const int m = std::min(MC_RHS, n_map - g);
    for (int r = 0; r < MC_RHS; ++r)
      for (int c = 0; c < 3; ++c) hp[3 * r + c] = r < m ? map_points[3 * (size_t)(g + r) + c] : 0.0;
    DS_CUDA(cudaMemcpyAsync(mp.p, hp.data(), hp.size() * sizeof(double), cudaMemcpyHostToDevice,
                            st));
    const long long total = (long long)n_pix * MC_RHS;
    k_mc_rhs<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(n_pix, MC_RHS, m, rec.p, mp.p, kc,
                                                             b.p);
    DS_CHECK_LAUNCH();
    DS_CUDA(cudaMemsetAsync(x.p, 0, (size_t)total * sizeof(double), st));
    rc = ds_batch_solve_mixed_dev(batch, &mpar, b.p, x.p, hit.data(), hconv.data(), nullptr,
                                  nullptr, nullptr);
    if (rc != DS_OK && rc != DS_ERR_NOT_CONVERGED) throw Error{rc, ctx->last_error};
    k_mc_dot<<<MC_RHS, 256, 0, st>>>(n_pix, MC_RHS, b.p, x.p, sig.p);
    DS_CHECK_LAUNCH();
    DS_CUDA(cudaMemcpyAsync(hs.data(), sig.p, MC_RHS * sizeof(double), cudaMemcpyDeviceToHost,
                            st));
    DS_CUDA(cudaStreamSynchronize(st));
    for (int r = 0; r < m; ++r) {
      success[g + r] = hconv[r] ? 1 : 0;
      iters[g + r] = hit[r];
      sigma_m[g + r] = hconv[r] ? hs[r] : 0.0;
    }
  }
}

}  // namespace

int ds_map_covar_diag(ds_context* ctx, int n_pix, const double* npixels, int n_map,
                      const double* map_points, const ds_kernel_params* kp,
                      const ds_pcg_params* pp, double* sigma_m, int* iters, int* success) {
  if (!ctx || !pp) return DS_ERR_ARG;
  if (kp && kp->eval == DS_EVAL_EXACT) {
    return guarded(ctx, [&] {
      require(n_pix > 0 && npixels, "bad pixel records");
      require(n_map >= 0 && (n_map == 0 || (map_points && sigma_m && iters && success)),
              "bad arguments");
      if (n_map > 0)
        map_covar_diag_batched(ctx, n_pix, npixels, n_map, map_points, *kp, *pp, sigma_m, iters,
                               success);
    });
  }
  ds_operator* op = nullptr;
  int rc = ds_operator_create(ctx, DS_FORM_SN, n_pix, npixels, kp, &op);
  if (rc != DS_OK) return rc;
  rc = guarded(ctx, [&] {
    require(n_map >= 0 && (n_map == 0 || (map_points && sigma_m && iters && success)),
            "bad arguments");
    require(pp->step_r > 0, "step_r must be > 0");
    if (n_map > 0) map_covar_diag_multi(op, n_map, map_points, *pp, sigma_m, iters, success);
  });
  ds_operator_destroy(op);
  return rc;
}

}  // extern "C"

extern "C" {

int ds_batch_create(ds_context* ctx, int form, int n_chunks, const int* chunk_sizes,
                    const double* records, const ds_kernel_params* kp, int n_rhs,
                    double inner_cutoff, ds_batch** out) {
  if (!ctx || !out) return DS_ERR_ARG;
  *out = nullptr;
  auto b = std::make_unique<ds_batch>();
  const int rc = guarded(ctx, [&] {
    require(form == DS_FORM_SN || form == DS_FORM_W, "form must be DS_FORM_SN or DS_FORM_W");
    require(n_chunks > 0 && chunk_sizes && records, "bad chunk arguments");
    require(n_rhs > 0 && n_rhs <= 1024, "n_rhs must be in [1, 1024]");
    long long total = 0;
    for (int c = 0; c < n_chunks; ++c) {
      require(chunk_sizes[c] > 0, "every chunk needs at least one record");
      total += chunk_sizes[c];
    }
    require(total < (1ll << 31), "too many records");
    const ds_kernel_params k = checked_kp(kp);
    require(k.eval == DS_EVAL_EXACT,
            "batched solves evaluate the exact kernel (eval = DS_EVAL_EXACT)");
    DS_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    b->ctx = ctx;
    b->form = form;
    b->n_chunks = n_chunks;
    b->n_rhs = n_rhs;
    b->n_total = (int)total;
    b->kc = make_consts(k);
    b->inner_cut = inner_cutoff > 0.0 ? inner_cutoff : DS_DEFAULT_INNER_CUTOFF;
    DevBuf<double> rec;
    upload(records, (size_t)total * 5, rec, st);
    batch_build(b.get(), rec.p, chunk_sizes);
  });
  if (rc != DS_OK) return rc;
  *out = b.release();
  return DS_OK;
}

void ds_batch_destroy(ds_batch* batch) { delete batch; }

int ds_batch_get_info(ds_batch* batch, ds_batch_info* info) {
  if (!batch || !info) return DS_ERR_ARG;
  info->n_chunks = batch->n_chunks;
  info->n_rhs = batch->n_rhs;
  info->n_total = batch->n_total;
  info->n_pad = batch->n_pad;
  info->n_tiles = batch->n_tiles;
  info->inner_tile_pairs = batch->pairs32_total;
  info->outer_tile_pairs = batch->pairs64_total;
  info->inner_evaluated = batch->eval32;
  info->outer_evaluated = batch->eval64;
  info->variant = batch->variant;
  info->rhs_block = batch->rb;
  info->graph_replays = batch->graph_replays;
  return DS_OK;
}

int ds_batch_set_variant(ds_batch* batch, int variant, int rhs_block) {
  if (!batch) return DS_ERR_ARG;
  return guarded(batch->ctx, [&] {
    if (variant == DS_BATCH_AUTO) {
      batch_autotune(batch, true, nullptr);
      return;
    }
    require(variant == DS_BATCH_CUDA_CORE || variant == DS_BATCH_TENSOR, "unknown batch variant");
    require(batch_variant_supported(batch, variant),
            "the tensor-core variant needs n_rhs % 16 == 0");
    if (rhs_block > 0 && variant == DS_BATCH_CUDA_CORE) {
      require(batch_rb_supported(batch->n_rhs, rhs_block), "unsupported RHS block");
      batch->rb = rhs_block;
    }
    batch->variant = variant;
    batch->tuned = true;
  });
}

static int batch_solve_common(ds_batch* batch, const ds_mixed_params* mp, const double* rhs,
                              double* x, int* iters, int* converged, int* n_updates,
                              double* rel_resid, double* seconds, bool host) {
  if (!batch || !mp) return DS_ERR_ARG;
  int status = DS_OK;
  const int rc = guarded(batch->ctx, [&] {
    require(rhs && x, "null vector");
    cudaStream_t st = batch->ctx->stream;
    const size_t nr = (size_t)batch->n_total * batch->n_rhs;
    const double* rd = rhs;
    double* xd = x;
    if (host) {
      upload(rhs, nr, batch->io_a, st);
      batch->io_b.alloc(nr);
      rd = batch->io_a.p;
      xd = batch->io_b.p;
    }
    std::vector<int> conv((size_t)batch->n_chunks * batch->n_rhs);
    batch_solve_dev(batch, *mp, rd, xd, iters, conv.data(), n_updates, rel_resid, seconds);
    if (converged) std::copy(conv.begin(), conv.end(), converged);
    if (host) {
      DS_CUDA(cudaMemcpyAsync(x, xd, nr * sizeof(double), cudaMemcpyDeviceToHost, st));
      DS_CUDA(cudaStreamSynchronize(st));
    }
    for (int v : conv)
      if (!v) status = DS_ERR_NOT_CONVERGED;
  });
  return rc != DS_OK ? rc : status;
}

int ds_batch_solve_mixed(ds_batch* batch, const ds_mixed_params* mp, const double* rhs,
                         double* x, int* iters, int* converged, int* n_updates,
                         double* rel_resid, double* seconds) {
  return batch_solve_common(batch, mp, rhs, x, iters, converged, n_updates, rel_resid, seconds,
                            true);
}

int ds_batch_solve_mixed_dev(ds_batch* batch, const ds_mixed_params* mp, const double* rhs,
                             double* x, int* iters, int* converged, int* n_updates,
                             double* rel_resid, double* seconds) {
  return batch_solve_common(batch, mp, rhs, x, iters, converged, n_updates, rel_resid, seconds,
                            false);
}

int ds_batch_product_f32_dev(ds_batch* batch, const double* p, double* q) {
  if (!batch) return DS_ERR_ARG;
  return guarded(batch->ctx, [&] {
    require(p && q, "null vector");
    batch_product_f32_dev(batch, p, q);
  });
}

}  // extern "C"
