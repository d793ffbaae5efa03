// FP64 matrix-free pair kernel: one CTA per row tile, one row per thread,
// looping over the row tile's culled column tiles.  Column coordinates and
// weights are staged in shared memory and read as broadcasts; the 200-knot
// table lives in shared memory.  Serves
//   * WFVector{SN,W}::A_product / A_residual (lib/wf_vector.cc:51-103,
//     196-251), with the CG dot d.q fused into the product epilogue;
//   * smp_product (lib/map.cc:20-43);
//   * sigma_m_noise_dom (lib/map_covar.cc:11-38).
// Roofline: FP64 pipe (about 16 FP64 instructions per pair in table mode,
// plus exp() in exact mode); no HBM traffic beyond the tiles (L2 resident).
#include "ds_device.cuh"

namespace ds {

namespace {

// Exact kernel without var_s, zero at and beyond the cutoff.
__device__ __forceinline__ double g_exact_fast(double dx, double dy, double dz,
                                               const KernelConsts& k, const double* tab) {
  const double arg = fma(k.c_perp, fma(dx, dx, dy * dy), k.c_para * (dz * dz));
  double g = 0.0;
  if (arg < k.exact_cut) g = exp_neg_f64(arg, tab);
  return g;
}

// Each warp's 32 rows form a k-d sub-tile with its own box; a staged column
// tile is four 32-column sub-tiles, and a warp skips every column sub-tile
// whose box is beyond the cutoff from its own (a warp-uniform branch).
template <int EVAL, int EPI, bool DOT>
__global__ void __launch_bounds__(TILE) k_pair_f64(KernelConsts kc, PairArgs a) {
  if (a.skip_flag && *a.skip_flag) return;
  // Warp-private staging of one 32-column sub-tile at a time: a warp loads
  // only the column sub-tiles its own row sub-tile interacts with, and the
  // warps of a CTA never wait for each other inside the loop.
  __shared__ double sw[TILE / 32][4][SUBTILE];
  __shared__ double tf[EVAL == DS_EVAL_TABLE ? TABLE_N : 32];
  __shared__ double red[TILE / 32];
  const int t = a.row_order ? a.row_order[blockIdx.x] : blockIdx.x;  // heaviest tiles first
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int i = t * TILE + tid;
  if (EVAL == DS_EVAL_TABLE) {
    for (int k = tid; k < TABLE_N; k += TILE) tf[k] = a.table[k];
  } else if (tid < 32) {
    tf[tid] = exp2(-(double)tid / 32.0);
  }
  __syncthreads();
  // var_s, folded into the column weights (squared for the S^2 sum)
  const double wscale = EPI == EPI_NOISE ? kc.var_s * kc.var_s : kc.var_s;
  const double xi = a.rx[i], yi = a.ry[i], zi = a.rz[i];
  double acc = 0.0;
  unsigned long long evaluated = 0;  // pairs this warp evaluates (profiling)
  double* sxw = sw[warp][0];
  double* syw = sw[warp][1];
  double* szw = sw[warp][2];
  double* suw = sw[warp][3];
  const int p0 = a.row_ptr[t], p1 = a.row_ptr[t + 1];
  for (int p = p0; p < p1; ++p) {
    const unsigned m = (a.mask[p] >> (4 * warp)) & 0xFu;  // this warp's row sub-tile
    if (!m) continue;
    const int ct = a.cols[p];
    for (int cs = 0; cs < TILE / SUBTILE; ++cs) {
      if (!((m >> cs) & 1u)) continue;
      const int j = ct * TILE + cs * SUBTILE + lane;
      __syncwarp();
      sxw[lane] = a.cx[j];
      syw[lane] = a.cy[j];
      szw[lane] = a.cz[j];
      if (EPI == EPI_PRODUCT || EPI == EPI_RESIDUAL)
        suw[lane] = wscale * (a.wr[j] * a.v[j]);
      else
        suw[lane] = wscale * a.v[j];
      __syncwarp();
      evaluated += SUBTILE * SUBTILE;
#pragma unroll 4
      for (int jj = 0; jj < SUBTILE; ++jj) {
        const double dx = xi - sxw[jj], dy = yi - syw[jj], dz = zi - szw[jj];
        double g = EVAL == DS_EVAL_TABLE ? gp_table_fast(dx, dy, dz, kc, tf)
                                         : g_exact_fast(dx, dy, dz, kc, tf);
        if (EPI == EPI_NOISE) g = g * g;
        acc = fma(g, suw[jj], acc);
      }
    }
  }
  if (a.prof_pairs && (tid & 31) == 0) atomicAdd(a.prof_pairs, evaluated);
  if (EPI == EPI_PRODUCT || EPI == EPI_RESIDUAL) {
    const double q = a.wl[i] * acc + a.e[i] * a.v[i];
    const double o = (EPI == EPI_RESIDUAL) ? a.b[i] - q : q;
    a.out[i] = o;
    if (DOT) {
      const double s = block_sum<TILE>(a.dotv[i] * o, red);
      if (tid == 0) a.dot_partial[t] = s;
      if (last_block_arrive(a.counter)) {
        const double dq = reduce_partials<TILE>(a.dot_partial, gridDim.x, 1, 0, red);
        if (tid == 0) {
          a.pcg->dq = dq;
          a.pcg->alpha = a.pcg->delta / dq;  // lib/pcg.h:37
          *a.counter = 0;
        }
      }
    }
  } else {
    const int dst = a.row_perm[i];
    if (dst >= 0) a.out[dst] = acc;
  }
}

template <int EVAL>
void launch_eval(const KernelConsts& kc, int epi, const PairArgs& a, cudaStream_t st) {
  const dim3 grid(a.n_row_tiles), block(TILE);
  switch (epi) {
    case EPI_PRODUCT:
      if (a.dot_partial)
        k_pair_f64<EVAL, EPI_PRODUCT, true><<<grid, block, 0, st>>>(kc, a);
      else
        k_pair_f64<EVAL, EPI_PRODUCT, false><<<grid, block, 0, st>>>(kc, a);
      break;
    case EPI_RESIDUAL:
      k_pair_f64<EVAL, EPI_RESIDUAL, false><<<grid, block, 0, st>>>(kc, a);
      break;
    case EPI_MAP:
      k_pair_f64<EVAL, EPI_MAP, false><<<grid, block, 0, st>>>(kc, a);
      break;
    case EPI_NOISE:
      k_pair_f64<EVAL, EPI_NOISE, false><<<grid, block, 0, st>>>(kc, a);
      break;
    default:
      throw Error{DS_ERR_ARG, "bad pair epilogue"};
  }
}

}  // namespace

void launch_pair_f64(const KernelConsts& kc, int epi, const PairArgs& a0, cudaStream_t st) {
  if (a0.n_row_tiles <= 0) return;
  PairArgs a = a0;
  cudaEvent_t ev = nullptr;
  const int kind = epi == EPI_MAP ? 2 : 0;
  if (a.prof && a.prof->enabled) {
    a.prof_pairs = a.prof->d_pairs + kind;
    a.prof->begin(st, &ev);
  } else {
    a.prof_pairs = nullptr;
  }
  if (kc.eval == DS_EVAL_TABLE)
    launch_eval<DS_EVAL_TABLE>(kc, epi, a, st);
  else
    launch_eval<DS_EVAL_EXACT>(kc, epi, a, st);
  DS_CHECK_LAUNCH();
  if (ev) a.prof->end(st, ev, kind);
}

long long& launch_counter() {
  static long long count = 0;
  return count;
}

cudaEvent_t Profiler::get_event() {
  if (!free_events.empty()) {
    cudaEvent_t e = free_events.back();
    free_events.pop_back();
    return e;
  }
  cudaEvent_t e;
  DS_CUDA(cudaEventCreate(&e));
  return e;
}

void Profiler::begin(cudaStream_t st, cudaEvent_t* ev) {
  *ev = get_event();
  DS_CUDA(cudaEventRecord(*ev, st));
}

void Profiler::end(cudaStream_t st, cudaEvent_t start, int kind) {
  cudaEvent_t e = get_event();
  DS_CUDA(cudaEventRecord(e, st));
  pending.push_back(Pending{start, e, kind});
}

void Profiler::collect() {
  // The events go back to the free list before they are read, so that an
  // error thrown from the checks never leaves an event in both lists.
  std::vector<Pending> work;
  work.swap(pending);
  for (const Pending& pr : work) {
    free_events.push_back(pr.start);
    free_events.push_back(pr.stop);
  }
  for (const Pending& pr : work) {
    DS_CUDA(cudaEventSynchronize(pr.stop));
    float t = 0.f;
    DS_CUDA(cudaEventElapsedTime(&t, pr.start, pr.stop));
    ms[pr.kind] += t;
    ++launches[pr.kind];
  }
}

Profiler::~Profiler() {
  for (auto& pr : pending) {
    cudaEventDestroy(pr.start);
    cudaEventDestroy(pr.stop);
  }
  for (auto e : free_events) cudaEventDestroy(e);
  if (d_pairs) cudaFree(d_pairs);
}

}  // namespace ds
