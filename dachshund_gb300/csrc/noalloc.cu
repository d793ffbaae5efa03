// ds_solve_pcg_noalloc: Jacobi-PCG for callers that cannot allocate device
// memory.  Everything the solve needs beyond the caller's own buffers lives
// in one file-scope device array of fixed size, kept until the process
// exits.  CUDA loads a library's device code lazily by default (since CUDA
// 12.2), so the array is reserved on a device when this file's code is first
// used there, i.e. by the first call on that device (which looks up the
// array's address), unless the process runs with CUDA_MODULE_LOADING=EAGER;
// callers should make that first call during their set-up.
//
// Compared with ds_solve_pcg it drops everything that needs memory of its
// own: no spatial sort (the radix sort needs temporary storage), no tile-pair
// list (its size is data dependent), no events and no pinned staging.  The
// matvec therefore visits every tile pair, which is why the size is capped.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <algorithm>
#include <mutex>

#include "ds_device.cuh"

namespace ds {
namespace {

constexpr int NA_MAX_N = 32768;       // largest n accepted (a multiple of TILE)
constexpr int NA_HIST = 8192;         // residual norms kept (later ones are not recorded)
constexpr int NA_VB = 256;
constexpr int NA_VGRID = 128;         // CTAs of the vector kernels
constexpr int NA_PARTIAL = 2 * NA_VGRID + NA_MAX_N / TILE;

struct NaState {
  double delta, delta_old, alpha, beta, dq, norm_r, tol_norm_b, pad0;
  int iter, max_iter, done, converged;
  unsigned int counter[4];
};

// Layout of the scratch array, in doubles.
constexpr size_t NA_OFF_X = 0;                              // x, y, z coordinates
constexpr size_t NA_OFF_COEF = NA_OFF_X + 3 * (size_t)NA_MAX_N;    // wl, e, b, pdiag
constexpr size_t NA_OFF_VEC = NA_OFF_COEF + 4 * (size_t)NA_MAX_N;  // xs, r, d, q, s
constexpr size_t NA_OFF_PART = NA_OFF_VEC + 5 * (size_t)NA_MAX_N;
constexpr size_t NA_OFF_HIST = NA_OFF_PART + NA_PARTIAL;
constexpr size_t NA_OFF_TABLE = NA_OFF_HIST + NA_HIST;
constexpr size_t NA_OFF_STATE = NA_OFF_TABLE + 256;
constexpr size_t NA_DOUBLES = NA_OFF_STATE + 16;  // 16 doubles hold NaState
static_assert(sizeof(NaState) <= 16 * sizeof(double), "state slot too small");

// The scratch: NA_DOUBLES * 8 bytes (about 3.3 MB), on every device that
// loads this library, for the life of the process.
static __device__ __align__(256) double ds_noalloc_scratch[NA_DOUBLES];

struct NaPtrs {
  double *x, *y, *z, *wl, *e, *b, *pdiag, *xs, *r, *d, *q, *s, *part, *hist, *table;
  NaState* st;
};

NaPtrs carve(double* base) {
  NaPtrs p;
  p.x = base + NA_OFF_X;
  p.y = p.x + NA_MAX_N;
  p.z = p.y + NA_MAX_N;
  p.wl = base + NA_OFF_COEF;
  p.e = p.wl + NA_MAX_N;
  p.b = p.e + NA_MAX_N;
  p.pdiag = p.b + NA_MAX_N;
  p.xs = base + NA_OFF_VEC;
  p.r = p.xs + NA_MAX_N;
  p.d = p.r + NA_MAX_N;
  p.q = p.d + NA_MAX_N;
  p.s = p.q + NA_MAX_N;
  p.part = base + NA_OFF_PART;
  p.hist = base + NA_OFF_HIST;
  p.table = base + NA_OFF_TABLE;
  p.st = reinterpret_cast<NaState*>(base + NA_OFF_STATE);
  return p;
}

// Records (caller order, device) -> SoA coordinates and operator
// coefficients; padding rows copy the last point and carry zero coefficients.
__global__ void k_na_load(int n, int n_pad, int form, double var_s, const double* __restrict__ rec,
                          const double* __restrict__ x0, NaPtrs p, int max_iter, double tol_norm_b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    NaState s{};
    s.max_iter = max_iter;
    s.tol_norm_b = tol_norm_b;
    *p.st = s;
  }
  if (i >= n_pad) return;
  const int src = i < n ? i : n - 1;
  const double* r = rec + (size_t)src * 5;
  p.x[i] = r[0];
  p.y[i] = r[1];
  p.z[i] = r[2];
  if (i >= n) {
    p.wl[i] = p.e[i] = p.b[i] = 0.0;
    p.pdiag[i] = 1.0;
    p.xs[i] = 0.0;
    return;
  }
  const double f = r[3];
  if (form == DS_FORM_SN) {
    p.wl[i] = 1.0;
    p.e[i] = f;
    p.pdiag[i] = __dadd_rn(var_s, f);
  } else {
    p.wl[i] = f;
    p.e[i] = 1.0;
    p.pdiag[i] = __dadd_rn(__dmul_rn(__dmul_rn(f, f), var_s), 1.0);
  }
  p.b[i] = r[4];
  p.xs[i] = x0[i];
}

// All-pairs operator: one CTA per 128-row tile, every column tile.
// epi 0: out = A v (+ v.out reduced into alpha = delta / (v.out)); 1: out = b - A v.
template <int EVAL>
__global__ void __launch_bounds__(TILE) k_na_matvec(KernelConsts kc, int n_tiles, int epi,
                                                    const double* __restrict__ v,
                                                    double* __restrict__ out, NaPtrs p) {
  if (p.st->done) return;
  __shared__ double sx[TILE], sy[TILE], sz[TILE], su[TILE];
  __shared__ double tf[TABLE_N];
  __shared__ double red[TILE / 32];
  const int t = blockIdx.x, tid = threadIdx.x, i = t * TILE + tid;
  for (int k = tid; k < TABLE_N; k += TILE) tf[k] = p.table[k];
  const double xi = p.x[i], yi = p.y[i], zi = p.z[i];
  double acc = 0.0;
  for (int c = 0; c < n_tiles; ++c) {
    const int j = c * TILE + tid;
    __syncthreads();
    sx[tid] = p.x[j];
    sy[tid] = p.y[j];
    sz[tid] = p.z[j];
    su[tid] = p.wl[j] * v[j];
    __syncthreads();
#pragma unroll 4
    for (int jj = 0; jj < TILE; ++jj)
      acc = fma(s_eval_f64<EVAL>(xi - sx[jj], yi - sy[jj], zi - sz[jj], kc, tf), su[jj], acc);
  }
  const double q = p.wl[i] * acc + p.e[i] * v[i];
  if (epi == 1) {
    out[i] = p.b[i] - q;
    return;
  }
  out[i] = q;
  const double s = block_sum<TILE>(v[i] * q, red);
  if (tid == 0) p.part[2 * NA_VGRID + t] = s;
  if (last_block_arrive(&p.st->counter[0])) {
    const double dq = reduce_partials<TILE>(p.part + 2 * NA_VGRID, gridDim.x, 1, 0, red);
    if (tid == 0) {
      p.st->dq = dq;
      p.st->alpha = p.st->delta / dq;
      p.st->counter[0] = 0;
    }
  }
}

// mode 0: normal step; 1: x update only; 2: precondition + dots after a
// full residual; 3: initial direction.
template <int MODE>
__global__ void __launch_bounds__(NA_VB) k_na_update(int n, NaPtrs p) {
  NaState* st = p.st;
  if (MODE != 3 && st->done) return;
  __shared__ double red[NA_VB / 32];
  const double alpha = (MODE == 0 || MODE == 1) ? st->alpha : 0.0;
  double rs = 0.0, rr = 0.0;
  for (int i = blockIdx.x * NA_VB + threadIdx.x; i < n; i += gridDim.x * NA_VB) {
    if (MODE == 0 || MODE == 1) p.xs[i] = fma(alpha, p.d[i], p.xs[i]);
    if (MODE == 1) continue;
    double ri = p.r[i];
    if (MODE == 0) {
      ri = fma(-alpha, p.q[i], ri);
      p.r[i] = ri;
    }
    const double si = ri / p.pdiag[i];
    if (MODE == 3)
      p.d[i] = si;
    else
      p.s[i] = si;
    rs = fma(ri, si, rs);
    rr = fma(ri, ri, rr);
  }
  if (MODE == 1) return;
  const double brs = block_sum<NA_VB>(rs, red);
  const double brr = block_sum<NA_VB>(rr, red);
  if (threadIdx.x == 0) {
    p.part[2 * blockIdx.x] = brs;
    p.part[2 * blockIdx.x + 1] = brr;
  }
  if (last_block_arrive(&st->counter[1])) {
    const double trs = reduce_partials<NA_VB>(p.part, gridDim.x, 2, 0, red);
    const double trr = reduce_partials<NA_VB>(p.part, gridDim.x, 2, 1, red);
    if (threadIdx.x == 0) {
      const double nr = sqrt(trr);
      if (MODE == 3) {
        st->delta = trs;
        st->iter = 0;
        st->norm_r = nr;
        p.hist[0] = nr;
        st->done = st->max_iter <= 1 ? 1 : 0;
      } else {
        st->delta_old = st->delta;
        st->delta = trs;
        st->beta = st->delta / st->delta_old;
        const int it = st->iter + 1;
        st->iter = it;
        st->norm_r = nr;
        if (it < NA_HIST) p.hist[it] = nr;
        if (nr <= st->tol_norm_b) {
          st->done = 1;
          st->converged = 1;
        } else if (it + 1 >= st->max_iter) {
          st->done = 1;
        }
      }
      st->counter[1] = 0;
    }
  }
}

__global__ void __launch_bounds__(NA_VB) k_na_direction(int n, NaPtrs p) {
  if (p.st->done) return;
  const double beta = p.st->beta;
  for (int i = blockIdx.x * NA_VB + threadIdx.x; i < n; i += gridDim.x * NA_VB)
    p.d[i] = fma(beta, p.d[i], p.s[i]);
}

// Solution out (caller order), times w in the W form.
__global__ void k_na_store(int n, int form, NaPtrs p, double* __restrict__ x) {
  for (int i = blockIdx.x * NA_VB + threadIdx.x; i < n; i += gridDim.x * NA_VB)
    x[i] = form == DS_FORM_W ? p.xs[i] * p.wl[i] : p.xs[i];
}

// |b| over the records, in record order on one thread (as norm_b does,
// lib/wf_vector.cc:105-112).
__global__ void k_na_norm_b(int n, const double* __restrict__ rec, double* out) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += rec[(size_t)i * 5 + 4] * rec[(size_t)i * 5 + 4];
  *out = sqrt(s);
}

// Per-device scratch address, looked up once per device.
std::mutex g_na_mutex;
double* g_na_base[64] = {nullptr};

}  // namespace
}  // namespace ds

using namespace ds;

extern "C" int ds_solve_pcg_noalloc(int form, int n, const double* records,
                                    const ds_kernel_params* kp, const ds_pcg_params* pp,
                                    double* x, ds_pcg_result* res, double* residual_norms,
                                    void* stream) {
  if (!kp || !pp || !records || !x) return DS_ERR_ARG;
  if (form != DS_FORM_SN && form != DS_FORM_W) return DS_ERR_ARG;
  if (n <= 0) return DS_ERR_ARG;
  if (n > NA_MAX_N) {
    fprintf(stderr,
            "[dachshund-gb300] ds_solve_pcg_noalloc: n = %d exceeds the fixed work space "
            "(at most %d pixels); use ds_solve_pcg\n",
            n, NA_MAX_N);
    return DS_ERR_ARG;
  }
  if (pp->step_r <= 0 || pp->max_iter < 0) return DS_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  try {
    const KernelConsts kc = make_consts(*kp);
    int dev = 0;
    DS_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return DS_ERR_NO_DEVICE;
    double* base;
    {
      std::lock_guard<std::mutex> lock(g_na_mutex);
      if (!g_na_base[dev]) {
        void* ptr = nullptr;
        DS_CUDA(cudaGetSymbolAddress(&ptr, ds_noalloc_scratch));
        g_na_base[dev] = static_cast<double*>(ptr);
      }
      base = g_na_base[dev];
    }
    const NaPtrs p = carve(base);
    const int n_tiles = (n + TILE - 1) / TILE, n_pad = n_tiles * TILE;

    // Table knots into the scratch (from the caller's table or built here).
    double table[TABLE_N];
    if (kp->table)
      for (int k = 0; k < TABLE_N; ++k) table[k] = kp->table[k];
    else
      host_table(table, nullptr);
    DS_CUDA(cudaMemcpyAsync(p.table, table, sizeof(table), cudaMemcpyHostToDevice, st));

    // |b| (record order), needed on the host for the tolerance.
    k_na_norm_b<<<1, 1, 0, st>>>(n, records, p.part);
    DS_CHECK_LAUNCH();
    double norm_b = 0.0;
    DS_CUDA(cudaMemcpyAsync(&norm_b, p.part, sizeof(double), cudaMemcpyDeviceToHost, st));
    DS_CUDA(cudaStreamSynchronize(st));

    const auto t0 = std::chrono::steady_clock::now();
    k_na_load<<<(n_pad + 255) / 256, 256, 0, st>>>(n, n_pad, form, kc.var_s, records, x, p,
                                                  pp->max_iter, pp->tol * norm_b);
    DS_CHECK_LAUNCH();
    ds_pcg_result r{};
    r.norm_b = norm_b;
    int status = DS_OK;
    auto matvec = [&](int epi, const double* v, double* out) {
      if (kc.eval == DS_EVAL_TABLE)
        k_na_matvec<DS_EVAL_TABLE><<<n_tiles, TILE, 0, st>>>(kc, n_tiles, epi, v, out, p);
      else
        k_na_matvec<DS_EVAL_EXACT><<<n_tiles, TILE, 0, st>>>(kc, n_tiles, epi, v, out, p);
      DS_CHECK_LAUNCH();
    };
    NaState h{};
    if (!(norm_b > 0.0)) {
      // lib/pcg.h:79-86: early return; the W form still scales x by w.
      puts("[WARNING] Requested PCG solve where |b| <= 0.0. Returning early.\n");
      status = DS_ERR_NORM_B;
    } else {
      matvec(1, p.xs, p.r);  // r = b - A x0
      k_na_update<3><<<NA_VGRID, NA_VB, 0, st>>>(n_pad, p);
      DS_CHECK_LAUNCH();
      constexpr int CHECK = 8;
      for (int it = 1; it < pp->max_iter; ++it) {
        matvec(0, p.d, p.q);
        if (it % pp->step_r == 0) {
          k_na_update<1><<<NA_VGRID, NA_VB, 0, st>>>(n_pad, p);
          DS_CHECK_LAUNCH();
          matvec(1, p.xs, p.r);
          k_na_update<2><<<NA_VGRID, NA_VB, 0, st>>>(n_pad, p);
        } else {
          k_na_update<0><<<NA_VGRID, NA_VB, 0, st>>>(n_pad, p);
        }
        DS_CHECK_LAUNCH();
        k_na_direction<<<NA_VGRID, NA_VB, 0, st>>>(n_pad, p);
        DS_CHECK_LAUNCH();
        if (it % CHECK == 0) {
          int done = 0;
          DS_CUDA(cudaMemcpyAsync(&done, &p.st->done, sizeof(int), cudaMemcpyDeviceToHost, st));
          DS_CUDA(cudaStreamSynchronize(st));
          if (done) break;
        }
      }
      DS_CUDA(cudaMemcpyAsync(&h, p.st, sizeof(h), cudaMemcpyDeviceToHost, st));
      DS_CUDA(cudaStreamSynchronize(st));
      r.final_norm = h.norm_r;
      r.n_inner = h.iter;
      if (pp->max_iter <= 1) {  // lib/pcg.h:117-158, as ds_solve_pcg
        r.success = pp->max_iter == 1 ? 0 : 1;
        r.num_iters = 1;
      } else if (h.converged) {
        r.success = 1;
        r.num_iters = h.iter;
      } else {
        r.success = 0;
        r.num_iters = pp->max_iter;
      }
      status = r.success ? DS_OK : DS_ERR_NOT_CONVERGED;
      if (!r.success) puts("[WARNING] PCG reached max iteration before stop condition.");
      if (residual_norms) {
        const int nh = std::min(h.iter + 1, NA_HIST);
        DS_CUDA(cudaMemcpyAsync(residual_norms, p.hist, nh * sizeof(double),
                                cudaMemcpyDeviceToHost, st));
      }
    }
    k_na_store<<<NA_VGRID, NA_VB, 0, st>>>(n, form, p, x);
    DS_CHECK_LAUNCH();
    DS_CUDA(cudaStreamSynchronize(st));
    r.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (res) *res = r;
    return status;
  } catch (const Error& e) {
    fprintf(stderr, "[dachshund-gb300] ds_solve_pcg_noalloc: %s\n", e.msg.c_str());
    return e.code;
  }
}
