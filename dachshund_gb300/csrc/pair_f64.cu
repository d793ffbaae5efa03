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

template <int EVAL, int EPI, bool DOT>
__global__ void __launch_bounds__(TILE) k_pair_f64(KernelConsts kc, PairArgs a) {
  if (a.skip_flag && *a.skip_flag) return;
  if (a.prof_pairs && blockIdx.x == 0 && threadIdx.x == 0)
    atomicAdd(a.prof_pairs, (unsigned long long)a.n_tile_pairs * TILE * TILE);
  __shared__ double sx[TILE], sy[TILE], sz[TILE], su[TILE];
  __shared__ double tf[EVAL == DS_EVAL_TABLE ? TABLE_N : 1];
  __shared__ double red[TILE / 32];
  const int t = blockIdx.x;
  const int tid = threadIdx.x;
  const int i = t * TILE + tid;
  if (EVAL == DS_EVAL_TABLE)
    for (int k = tid; k < TABLE_N; k += TILE) tf[k] = a.table[k];
  const double xi = a.rx[i], yi = a.ry[i], zi = a.rz[i];
  double acc = 0.0;
  const int p0 = a.row_ptr[t], p1 = a.row_ptr[t + 1];
  for (int p = p0; p < p1; ++p) {
    const int j = a.cols[p] * TILE + tid;
    __syncthreads();
    sx[tid] = a.cx[j];
    sy[tid] = a.cy[j];
    sz[tid] = a.cz[j];
    if (EPI == EPI_PRODUCT || EPI == EPI_RESIDUAL)
      su[tid] = a.wr[j] * a.v[j];
    else
      su[tid] = a.v[j];
    __syncthreads();
#pragma unroll 4
    for (int jj = 0; jj < TILE; ++jj) {
      double S = s_eval_f64<EVAL>(xi - sx[jj], yi - sy[jj], zi - sz[jj], kc, tf);
      if (EPI == EPI_NOISE) S = S * S;
      acc = fma(S, su[jj], acc);
    }
  }
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
  if (a.prof && a.prof->enabled) {
    a.prof_pairs = a.prof->d_pairs;
    a.prof->begin(st, &ev);
  } else {
    a.prof_pairs = nullptr;
  }
  if (kc.eval == DS_EVAL_TABLE)
    launch_eval<DS_EVAL_TABLE>(kc, epi, a, st);
  else
    launch_eval<DS_EVAL_EXACT>(kc, epi, a, st);
  DS_CHECK_LAUNCH();
  if (ev) a.prof->end(st, ev, 0);
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
  for (auto& pr : pending) {
    DS_CUDA(cudaEventSynchronize(pr.stop));
    float t = 0.f;
    DS_CUDA(cudaEventElapsedTime(&t, pr.start, pr.stop));
    ms[pr.kind] += t;
    ++launches[pr.kind];
    free_events.push_back(pr.start);
    free_events.push_back(pr.stop);
  }
  pending.clear();
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
