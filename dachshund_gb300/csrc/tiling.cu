// Spatial sorting, tiling and tile-pair culling.
//
// The reference evaluates every (i, j) pair of every matvec
// (lib/wf_vector.cc:51-74) even where the table kernel is exactly zero
// (lib/signal_covar.h:60-62).  Here points are sorted along a 3-D Morton curve
// of their coordinates scaled by the correlation lengths, cut into tiles of
// TILE consecutive points, and a tile pair is kept only when the nearest
// corners of the two bounding boxes are inside the kernel's cutoff.  Every
// skipped pair therefore has S_ij == 0 (table) or S_ij < var_s exp(-cutoff)
// (exact), and the kept relation is symmetric, so A stays symmetric.
#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <numeric>

#include "ds_internal.cuh"

namespace ds {

void host_table(double* table, double* dx_inv) {
  // SignalCovarParams ctor, lib/signal_covar.h:25-40.
  const double fx_max = 4.0 * 4.0 / 2.0;
  const double ft_dx = fx_max / (TABLE_N - 1);
  if (dx_inv) *dx_inv = 1.0 / ft_dx;
  if (table)
    for (int i = 0; i < TABLE_N; ++i) table[i] = std::exp(-(ft_dx * i));
}

KernelConsts make_consts(const ds_kernel_params& kp) {
  require(kp.var_s >= 0.0 && std::isfinite(kp.var_s), "var_s must be finite and >= 0");
  require(kp.l_perp > 0.0 && kp.l_para > 0.0, "correlation lengths must be > 0");
  require(kp.eval == DS_EVAL_TABLE || kp.eval == DS_EVAL_EXACT, "unknown eval mode");
  KernelConsts k{};
  k.var_s = kp.var_s;
  k.c_perp = 1.0 / (2.0 * kp.l_perp * kp.l_perp);
  k.c_para = 1.0 / (2.0 * kp.l_para * kp.l_para);
  host_table(nullptr, &k.dx_inv);
  k.exact_cut = kp.exact_cutoff > 0.0 ? kp.exact_cutoff : DS_DEFAULT_EXACT_CUTOFF;
  k.eval = kp.eval;
  // Table: S == 0 once xx = arg * dx_inv reaches TABLE_N - 1.
  const double cut = kp.eval == DS_EVAL_TABLE ? (TABLE_N - 1) / k.dx_inv : k.exact_cut;
  k.cull_arg = cut * (1.0 + 1e-9);
  return k;
}

namespace {

constexpr int BLK = 256;

__global__ void k_bbox_partial(const double* __restrict__ rec, int n, int stride,
                               double* __restrict__ part) {
  double lo[3] = {INFINITY, INFINITY, INFINITY};
  double hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    for (int c = 0; c < 3; ++c) {
      const double v = rec[(size_t)i * stride + c];
      if (v != v) {  // NaN (fmin and fmax would skip it): the bounds go infinite
        lo[c] = -INFINITY;
        hi[c] = INFINITY;
      }
      lo[c] = fmin(lo[c], v);
      hi[c] = fmax(hi[c], v);
    }
  }
  __shared__ double sm[6][BLK];
  for (int c = 0; c < 3; ++c) {
    sm[c][threadIdx.x] = lo[c];
    sm[3 + c][threadIdx.x] = hi[c];
  }
  __syncthreads();
  for (int s = BLK / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      for (int c = 0; c < 3; ++c) {
        sm[c][threadIdx.x] = fmin(sm[c][threadIdx.x], sm[c][threadIdx.x + s]);
        sm[3 + c][threadIdx.x] = fmax(sm[3 + c][threadIdx.x], sm[3 + c][threadIdx.x + s]);
      }
    }
    __syncthreads();
  }
  if (threadIdx.x < 6) part[blockIdx.x * 6 + threadIdx.x] = sm[threadIdx.x][0];
}

__device__ __forceinline__ uint32_t spread3(uint32_t v) {
  // 10 bits -> every third bit of 30.
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__global__ void k_morton(const double* __restrict__ rec, int n, int stride, double lx,
                         double ly, double lz, double sx, double sy, double sz,
                         double inv_h, uint32_t* __restrict__ keys, int* __restrict__ idx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double* p = rec + (size_t)i * stride;
  auto q = [&](double v, double lo, double s) {
    double c = (v - lo) * s * inv_h;
    c = fmin(fmax(c, 0.0), 1023.0);
    return (uint32_t)c;
  };
  const uint32_t qx = q(p[0], lx, sx), qy = q(p[1], ly, sy), qz = q(p[2], lz, sz);
  keys[i] = spread3(qx) | (spread3(qy) << 1) | (spread3(qz) << 2);
  idx[i] = i;
}

__global__ void k_gather_points(const double* __restrict__ rec, int n, int n_pad, int stride,
                                const int* __restrict__ sorted_idx, double* __restrict__ x,
                                double* __restrict__ y, double* __restrict__ z,
                                int* __restrict__ perm) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pad) return;
  const int src = sorted_idx[i < n ? i : n - 1];
  const double* p = rec + (size_t)src * stride;
  x[i] = p[0];
  y[i] = p[1];
  z[i] = p[2];
  perm[i] = i < n ? src : -1;
}

// Boxes of consecutive groups of blockDim.x (TILE or SUBTILE) sorted points.
__global__ void k_tile_boxes(const double* __restrict__ x, const double* __restrict__ y,
                             const double* __restrict__ z, double* __restrict__ box) {
  const int t = blockIdx.x;
  const int i = t * blockDim.x + threadIdx.x;
  __shared__ double sm[6][TILE];
  sm[0][threadIdx.x] = x[i];
  sm[1][threadIdx.x] = y[i];
  sm[2][threadIdx.x] = z[i];
  sm[3][threadIdx.x] = x[i];
  sm[4][threadIdx.x] = y[i];
  sm[5][threadIdx.x] = z[i];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      for (int c = 0; c < 3; ++c) {
        sm[c][threadIdx.x] = fmin(sm[c][threadIdx.x], sm[c][threadIdx.x + s]);
        sm[3 + c][threadIdx.x] = fmax(sm[3 + c][threadIdx.x], sm[3 + c][threadIdx.x + s]);
      }
    }
    __syncthreads();
  }
  if (threadIdx.x < 6) box[t * 6 + threadIdx.x] = sm[threadIdx.x][0];
}

// ---- k-d partition -----------------------------------------------------

// Working points of the partition: the scaled coordinates in FP32 and the
// record index (its bits in w), permuted with the keys by each level's sort,
// so the levels read them contiguously (the axis choices need no more than
// FP32; the tiles' boxes are formed afterwards from the FP64 coordinates).
static_assert(SUBTILE == 32, "one warp per unit");
__global__ void k_kd_points(const double* __restrict__ rec, int n, int stride,
                            const int* __restrict__ idx, double sx, double sy, double sz,
                            float4* __restrict__ pv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int r = idx[i];
  const double* p = rec + (size_t)r * stride;
  pv[i] = make_float4((float)(p[0] * sx), (float)(p[1] * sy), (float)(p[2] * sz),
                      __int_as_float(r));
}

__global__ void k_kd_index(int n, const float4* __restrict__ pv, int* __restrict__ idx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) idx[i] = __float_as_int(pv[i].w);
}

// Boxes (lo x y z, hi x y z) of every SUBTILE-point unit of the current
// order: one warp per unit.
__global__ void k_unit_boxes(int n, int nu, const float4* __restrict__ pv,
                             float* __restrict__ box) {
  const int u = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (u >= nu) return;
  const int i = u * SUBTILE + lane;
  float lx = INFINITY, ly = INFINITY, lz = INFINITY, hx = -INFINITY, hy = -INFINITY,
        hz = -INFINITY;
  if (i < n) {
    const float4 q = pv[i];
    lx = hx = q.x;
    ly = hy = q.y;
    lz = hz = q.z;
  }
  for (int o = 16; o > 0; o >>= 1) {
    lx = fminf(lx, __shfl_xor_sync(0xffffffffu, lx, o));
    ly = fminf(ly, __shfl_xor_sync(0xffffffffu, ly, o));
    lz = fminf(lz, __shfl_xor_sync(0xffffffffu, lz, o));
    hx = fmaxf(hx, __shfl_xor_sync(0xffffffffu, hx, o));
    hy = fmaxf(hy, __shfl_xor_sync(0xffffffffu, hy, o));
    hz = fmaxf(hz, __shfl_xor_sync(0xffffffffu, hz, o));
  }
  if (lane == 0) {
    float* b = box + (size_t)u * 6;
    b[0] = lx;
    b[1] = ly;
    b[2] = lz;
    b[3] = hx;
    b[4] = hy;
    b[5] = hz;
  }
}

// node_of_unit for the units of every node of a level (one CTA per node).
__global__ void k_node_units(const int2* __restrict__ nodes, int* __restrict__ node_of_unit) {
  const int k = blockIdx.x;
  const int2 nd = nodes[k];
  for (int u = nd.x + threadIdx.x; u < nd.y; u += blockDim.x) node_of_unit[u] = k;
}

// Split axis of every node of a level with at least two units (TPN threads
// per node: a warp, or a whole CTA where the nodes hold thousands of
// units): the longest side of the union of its unit boxes (the first of
// equal sides), else -1, and the map of that side onto the key's cb
// coordinate bits (range[k] = (lo, (2^cb - 1) / (hi - lo))).  Min and max
// are exact, so the order of the reduction does not matter.
template <int TPN>
__global__ void __launch_bounds__(BLK) k_node_axis(int nn, const int2* __restrict__ nodes,
                                                   const float* __restrict__ box, int cb,
                                                   int* __restrict__ node_axis,
                                                   double2* __restrict__ range) {
  static_assert(TPN == 32 || TPN == BLK, "a warp or the CTA per node");
  __shared__ float red[BLK / 32][6];
  const int k = blockIdx.x * (BLK / TPN) + threadIdx.x / TPN;
  const int g = threadIdx.x % TPN, lane = threadIdx.x & 31;
  const bool live = k < nn;
  const int2 nd = live ? nodes[k] : make_int2(0, 0);
  if (TPN == 32 && (!live || nd.y - nd.x < 2)) {  // warp-uniform
    if (live && lane == 0) node_axis[k] = -1;
    return;
  }
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
#pragma unroll 4
  for (int u = nd.x + g; u < nd.y; u += TPN) {
    const float* b = box + (size_t)u * 6;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      lo[c] = fminf(lo[c], b[c]);
      hi[c] = fmaxf(hi[c], b[3 + c]);
    }
  }
#pragma unroll
  for (int c = 0; c < 3; ++c)
    for (int o = 16; o > 0; o >>= 1) {
      lo[c] = fminf(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
      hi[c] = fmaxf(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
    }
  if (TPN > 32) {  // the CTA's warps (one node per CTA)
    const int w = threadIdx.x >> 5;
    if (lane == 0)
      for (int c = 0; c < 3; ++c) {
        red[w][c] = lo[c];
        red[w][3 + c] = hi[c];
      }
    __syncthreads();
    if (threadIdx.x == 0)
      for (int w2 = 1; w2 < BLK / 32; ++w2)
        for (int c = 0; c < 3; ++c) {
          lo[c] = fminf(lo[c], red[w2][c]);
          hi[c] = fmaxf(hi[c], red[w2][3 + c]);
        }
  }
  if (g == 0 && live) {
    if (nd.y - nd.x < 2) {
      node_axis[k] = -1;
      return;
    }
    const float e0 = hi[0] - lo[0], e1 = hi[1] - lo[1], e2 = hi[2] - lo[2];
    int ax = 0;
    float ext = e0, l = lo[0];
    if (e1 > ext) {
      ax = 1;
      ext = e1;
      l = lo[1];
    }
    if (e2 > ext) {
      ax = 2;
      ext = e2;
      l = lo[2];
    }
    node_axis[k] = ax;
    range[k] = make_double2(l, ext > 0.f ? (double)((1u << cb) - 1u) / (double)ext : 0.0);
  }
}

// key = node << cb | the point's coordinate along the node's split axis
// mapped onto cb bits over the node's range (0 for nodes that are already
// leaves).  A node of a level with nn nodes holds at most 32 n / nn points
// and gets 2^cb >= 2^32 / nn levels, so only coordinates closer than the
// node's extent / 2^cb share a key (and keep their order: the sort is stable).
__global__ void k_kd_keys(int n, const float4* __restrict__ pv,
                          const int* __restrict__ node_of_unit, const int* __restrict__ node_axis,
                          const double2* __restrict__ range, int cb,
                          unsigned int* __restrict__ keys) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int node = node_of_unit[i / SUBTILE];
  const int axis = node_axis[node];
  unsigned int u = 0;
  if (axis >= 0) {
    const float4 q = pv[i];
    const float v = axis == 0 ? q.x : (axis == 1 ? q.y : q.z);
    const double2 rg = range[node];
    const double f = ((double)v - rg.x) * rg.y;
    const unsigned int top = (1u << cb) - 1u;
    u = f <= 0.0 ? 0u : (f >= (double)top ? top : (unsigned int)f);
  }
  keys[i] = ((unsigned int)node << cb) | u;
}

__global__ void k_iota(int n, int* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = i;
}

// Culling test of two boxes: c_perp (dx^2 + dy^2) + c_para dz^2 < cut at the
// nearest corners, in FP32 (FP64 runs at 2 FMA per clock per SM on GB300).
// The boxes are rounded outward, every gap, product and sum is rounded down
// and c_perp, c_para down, cut up, so the FP32 argument never exceeds the
// exact one: a pair that interacts is never culled (a pair within rounding of
// the cutoff may be kept).  The test is symmetric in the two boxes, so the
// kept relation stays symmetric.
struct CullConsts {
  float c_perp, c_para, cut;
};

__device__ __forceinline__ bool tiles_interact(const float* __restrict__ bi,
                                               const float* __restrict__ bj,
                                               const CullConsts& k) {
  const float dx = fmaxf(0.f, fmaxf(__fsub_rd(bi[0], bj[3]), __fsub_rd(bj[0], bi[3])));
  const float dy = fmaxf(0.f, fmaxf(__fsub_rd(bi[1], bj[4]), __fsub_rd(bj[1], bi[4])));
  const float dz = fmaxf(0.f, fmaxf(__fsub_rd(bi[2], bj[5]), __fsub_rd(bj[2], bi[5])));
  const float perp = __fmaf_rd(dy, dy, __fmul_rd(dx, dx));
  return __fmaf_rd(k.c_perp, perp, __fmul_rd(k.c_para, __fmul_rd(dz, dz))) < k.cut;
}

float f32_down(double v) {
  float f = (float)v;
  if ((double)f > v) f = std::nextafter(f, -INFINITY);
  return f;
}

float f32_up(double v) {
  float f = (float)v;
  if ((double)f < v) f = std::nextafter(f, INFINITY);
  return f;
}

CullConsts cull_consts(const KernelConsts& kc) {
  return CullConsts{f32_down(kc.c_perp), f32_down(kc.c_para), f32_up(kc.cull_arg)};
}

// Outward FP32 copies of n boxes (6 values each: lo x, y, z, hi x, y, z).
__global__ void k_box_f32(long long n6, const double* __restrict__ b, float* __restrict__ f) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n6) return;
  f[i] = (i % 6) < 3 ? __double2float_rd(b[i]) : __double2float_ru(b[i]);
}

// Union boxes of consecutive groups of 32 column tiles (k-d order keeps a
// group spatially compact).  A row tile that does not interact with a
// group's box interacts with none of its tiles (the distance to a union box
// is at most the distance to each member), so the pair search tests group
// boxes first and tile boxes only inside interacting groups: the same kept
// pairs as testing every tile box.
constexpr int PGROUP = 32;

__global__ void k_group_boxes(int n_col, const float* __restrict__ cbox,
                              float* __restrict__ gbox) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int n_groups = (n_col + PGROUP - 1) / PGROUP;
  if (g >= n_groups) return;
  float b[6];
  for (int c = 0; c < 6; ++c) b[c] = cbox[(size_t)g * PGROUP * 6 + c];
  for (int j = g * PGROUP + 1; j < min(n_col, (g + 1) * PGROUP); ++j)
    for (int c = 0; c < 3; ++c) {
      b[c] = fminf(b[c], cbox[(size_t)j * 6 + c]);
      b[c + 3] = fmaxf(b[c + 3], cbox[(size_t)j * 6 + c + 3]);
    }
  for (int c = 0; c < 6; ++c) gbox[(size_t)g * 6 + c] = b[c];
}

// Per row tile (one CTA of BLK threads): for every column group the ballot
// of its interacting tiles (0 when the group box does not interact), in
// shared memory gm[n_groups].  FILL then writes the kept columns in
// ascending order at row_ptr[r]; otherwise counts[r] = their number.
template <bool FILL>
__global__ void k_pair_search(const float* __restrict__ rbox, const float* __restrict__ cbox,
                              const float* __restrict__ gbox, int n_col, CullConsts kc,
                              int* __restrict__ counts, const int* __restrict__ row_ptr,
                              int* __restrict__ cols) {
  extern __shared__ unsigned gm[];  // [n_groups]
  __shared__ int wsum[BLK / 32];
  const int r = blockIdx.x;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int n_groups = (n_col + PGROUP - 1) / PGROUP;
  float bi[6];
  for (int c = 0; c < 6; ++c) bi[c] = rbox[(size_t)r * 6 + c];
  int cnt = 0;
  for (int g = wid; g < n_groups; g += BLK / 32) {
    const bool gi = tiles_interact(bi, gbox + (size_t)g * 6, kc);
    unsigned m = 0;
    if (gi) {  // warp-uniform
      const int j = g * PGROUP + lane;
      m = __ballot_sync(0xffffffffu,
                        j < n_col && tiles_interact(bi, cbox + (size_t)j * 6, kc));
    }
    if (lane == 0) gm[g] = m;
    cnt += __popc(m);
  }
  if (lane == 0) wsum[wid] = cnt;
  __syncthreads();
  if (!FILL) {
    if (threadIdx.x == 0) {
      int t = 0;
      for (int w = 0; w < BLK / 32; ++w) t += wsum[w];
      counts[r] = t;
    }
    return;
  }
  // ascending order: group offsets by a scan over the groups (warp 0), then
  // every warp writes its groups' columns
  __shared__ int base;
  if (wid == 0) {
    int run = 0;
    for (int g0 = 0; g0 < n_groups; g0 += 32) {
      const int g = g0 + lane;
      const int c = g < n_groups ? __popc(gm[g]) : 0;
      int incl = c;
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
      }
      const int excl = run + incl - c;
      run += __shfl_sync(0xffffffffu, incl, 31);
      // offsets go to the second half of gm
      if (g < n_groups) gm[n_groups + g] = (unsigned)excl;
    }
    if (lane == 0) base = row_ptr[r];
  }
  __syncthreads();
  for (int g = wid; g < n_groups; g += BLK / 32) {
    const unsigned m = gm[g];
    if (!m) continue;
    if ((m >> lane) & 1u)
      cols[base + (int)gm[n_groups + g] + __popc(m & ((1u << lane) - 1u))] = g * PGROUP + lane;
  }
}

// Sub-tile interaction masks of every kept tile pair: bit 4 k + w for row
// sub-tile k and column sub-tile w.
__global__ void k_pair_mask(int n_rows, const int* __restrict__ row_ptr,
                            const int* __restrict__ cols, const float* __restrict__ rsbox,
                            const float* __restrict__ csbox, CullConsts kc,
                            unsigned short* __restrict__ mask) {
  const int r = blockIdx.x;
  if (r >= n_rows) return;
  float rb[4][6];
  for (int k = 0; k < 4; ++k)
    for (int c = 0; c < 6; ++c) rb[k][c] = rsbox[((size_t)r * 4 + k) * 6 + c];
  for (int p = row_ptr[r] + threadIdx.x; p < row_ptr[r + 1]; p += blockDim.x) {
    const int ct = cols[p];
    unsigned m = 0;
    for (int w = 0; w < 4; ++w) {
      const float* cb = csbox + ((size_t)ct * 4 + w) * 6;
      for (int k = 0; k < 4; ++k)
        if (tiles_interact(rb[k], cb, kc)) m |= 1u << (4 * k + w);
    }
    mask[p] = (unsigned short)m;
  }
}

}  // namespace

// Balanced k-d partition.  Nodes cover whole SUBTILE-point units [u0, u1);
// a node larger than a tile splits at a tile boundary near its middle, a node
// within a tile splits at a unit boundary, so every TILE-point tile is a k-d
// node and its four SUBTILE-point quarters are k-d nodes too (compact boxes
// for each warp's rows).  Each level is one stable radix sort of 32-bit keys
// (node, coordinate along the node's longest scaled axis) that carries the
// points' FP32 coordinates and record indices, which keeps every node's
// points contiguous.  idx (sorted position -> record) is updated in place.
void kd_partition(const PointSet& ps, const double* d_rec, int n, int stride, double sx,
                  double sy, double sz, DevBuf<int>& idx, cudaStream_t st) {
  (void)ps;
  constexpr int UPT = TILE / SUBTILE;  // units per tile
  const int nu = (n + SUBTILE - 1) / SUBTILE;
  // The nodes of every level follow from the unit counts alone (only the
  // split axes depend on the points): all levels are listed here and copied
  // once; each level then runs on the device without a host round trip.
  std::vector<int2> all_nodes;
  std::vector<size_t> level_off;
  {
    std::vector<int2> nodes{make_int2(0, nu)};
    for (;;) {
      bool any = false;
      for (auto& nd : nodes) any |= (nd.y - nd.x) >= 2;
      if (!any) break;
      level_off.push_back(all_nodes.size());
      all_nodes.insert(all_nodes.end(), nodes.begin(), nodes.end());
      std::vector<int2> next;
      next.reserve(nodes.size() * 2);
      for (auto& nd : nodes) {
        const int len = nd.y - nd.x;
        if (len < 2) {
          next.push_back(nd);
        } else {
          const int ntile = (len + UPT - 1) / UPT;
          const int um = ntile >= 2 ? nd.x + UPT * (ntile / 2) : nd.x + len / 2;
          next.push_back(make_int2(nd.x, um));
          next.push_back(make_int2(um, nd.y));
        }
      }
      nodes.swap(next);
    }
    level_off.push_back(all_nodes.size());
  }
  const int n_levels = (int)level_off.size() - 1;
  if (n_levels <= 0) return;
  DevBuf<int2> d_nodes;
  d_nodes.alloc(all_nodes.size());
  DS_CUDA(cudaMemcpyAsync(d_nodes.p, all_nodes.data(), all_nodes.size() * sizeof(int2),
                          cudaMemcpyHostToDevice, st));
  DevBuf<float> box;
  box.alloc((size_t)nu * 6);
  DevBuf<int> d_not, d_axis;
  DevBuf<double2> d_range;
  d_not.alloc(nu);
  d_axis.alloc(level_off[n_levels] - level_off[n_levels - 1]);
  d_range.alloc(level_off[n_levels] - level_off[n_levels - 1]);
  DevBuf<float4> pv, pv2;
  pv.alloc(n);
  pv2.alloc(n);
  DevBuf<unsigned int> keys, keys2;
  keys.alloc(n);
  keys2.alloc(n);
  DevBuf<unsigned char> tmp;
  k_kd_points<<<(n + BLK - 1) / BLK, BLK, 0, st>>>(d_rec, n, stride, idx.p, sx, sy, sz, pv.p);
  DS_CHECK_LAUNCH();
  constexpr int WPB = BLK / 32;  // warps per CTA
  for (int level = 0; level < n_levels; ++level) {
    const int nn = (int)(level_off[level + 1] - level_off[level]);
    const int2* nodes = d_nodes.p + level_off[level];
    k_node_units<<<nn, 128, 0, st>>>(nodes, d_not.p);
    DS_CHECK_LAUNCH();
    k_unit_boxes<<<(nu + WPB - 1) / WPB, BLK, 0, st>>>(n, nu, pv.p, box.p);
    DS_CHECK_LAUNCH();
    int node_bits = 1;
    while ((1ull << node_bits) < (unsigned long long)nn) ++node_bits;
    const int cb = 32 - node_bits;  // coordinate bits of the key
    if (nu >= 256 * nn)  // thousands of units per node: a CTA per node
      k_node_axis<BLK><<<nn, BLK, 0, st>>>(nn, nodes, box.p, cb, d_axis.p, d_range.p);
    else
      k_node_axis<32><<<(nn + WPB - 1) / WPB, BLK, 0, st>>>(nn, nodes, box.p, cb, d_axis.p,
                                                            d_range.p);
    DS_CHECK_LAUNCH();
    k_kd_keys<<<(n + BLK - 1) / BLK, BLK, 0, st>>>(n, pv.p, d_not.p, d_axis.p, d_range.p, cb,
                                                  keys.p);
    DS_CHECK_LAUNCH();
    size_t tmp_bytes = 0;
    DS_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys.p, keys2.p, pv.p, pv2.p, n,
                                            0, 32, st));
    if (tmp.n < tmp_bytes) tmp.alloc(tmp_bytes);
    DS_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, keys.p, keys2.p, pv.p, pv2.p, n, 0,
                                            32, st));
    std::swap(pv.p, pv2.p);
  }
  k_kd_index<<<(n + BLK - 1) / BLK, BLK, 0, st>>>(n, pv.p, idx.p);
  DS_CHECK_LAUNCH();
}

void point_bbox(const double* d_rec, int n, int stride, double lo[3], double hi[3],
                cudaStream_t st) {
  require(n > 0, "point count must be > 0");
  const int nb = std::min(1216, (n + BLK - 1) / BLK);  // 8 CTAs per SM of 152
  DevBuf<double> part;
  part.alloc((size_t)nb * 6);
  k_bbox_partial<<<nb, BLK, 0, st>>>(d_rec, n, stride, part.p);
  DS_CHECK_LAUNCH();
  std::vector<double> hp((size_t)nb * 6);
  DS_CUDA(cudaMemcpyAsync(hp.data(), part.p, hp.size() * sizeof(double),
                          cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaStreamSynchronize(st));
  for (int c = 0; c < 3; ++c) {
    lo[c] = INFINITY;
    hi[c] = -INFINITY;
  }
  for (int b = 0; b < nb; ++b)
    for (int c = 0; c < 3; ++c) {
      lo[c] = std::min(lo[c], hp[b * 6 + c]);
      hi[c] = std::max(hi[c], hp[b * 6 + 3 + c]);
    }
  for (int c = 0; c < 3; ++c)
    require(std::isfinite(lo[c]) && std::isfinite(hi[c]), "non-finite coordinates");
}

void build_point_set(PointSet& ps, const double* d_rec, int n, int stride, double sx,
                     double sy, double sz, cudaStream_t st, int order) {
  require(n > 0, "point count must be > 0");
  ps.n = n;
  ps.n_tiles = (n + TILE - 1) / TILE;
  ps.n_pad = ps.n_tiles * TILE;

  // Bounding box of all points.
  double lo[3], hi[3];
  point_bbox(d_rec, n, stride, lo, hi, st);
  const double ext = std::max({(hi[0] - lo[0]) * sx, (hi[1] - lo[1]) * sy,
                               (hi[2] - lo[2]) * sz, 1e-300});
  const double inv_h = 1023.0 / ext;

  // Morton keys and a stable radix sort of (key, index).
  DevBuf<uint32_t> keys, keys2;
  DevBuf<int> idx, idx2;
  keys.alloc(n);
  keys2.alloc(n);
  idx.alloc(n);
  idx2.alloc(n);
  k_morton<<<(n + BLK - 1) / BLK, BLK, 0, st>>>(d_rec, n, stride, lo[0], lo[1], lo[2], sx, sy,
                                                sz, inv_h, keys.p, idx.p);
  DS_CHECK_LAUNCH();
  size_t tmp_bytes = 0;
  DS_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys.p, keys2.p, idx.p, idx2.p, n,
                                          0, 30, st));
  DevBuf<unsigned char> tmp;
  tmp.alloc(std::max<size_t>(tmp_bytes, 1));
  DS_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, keys.p, keys2.p, idx.p, idx2.p, n, 0,
                                          30, st));
  if (order == ORDER_KD && ps.n_tiles > 1) kd_partition(ps, d_rec, n, stride, sx, sy, sz, idx2, st);

  ps.x.alloc(ps.n_pad);
  ps.y.alloc(ps.n_pad);
  ps.z.alloc(ps.n_pad);
  ps.perm.alloc(ps.n_pad);
  ps.box.alloc((size_t)ps.n_tiles * 6);
  k_gather_points<<<(ps.n_pad + BLK - 1) / BLK, BLK, 0, st>>>(d_rec, n, ps.n_pad, stride, idx2.p,
                                                              ps.x.p, ps.y.p, ps.z.p, ps.perm.p);
  DS_CHECK_LAUNCH();
  k_tile_boxes<<<ps.n_tiles, TILE, 0, st>>>(ps.x.p, ps.y.p, ps.z.p, ps.box.p);
  DS_CHECK_LAUNCH();
  ps.sbox.alloc((size_t)(ps.n_pad / SUBTILE) * 6);
  k_tile_boxes<<<ps.n_pad / SUBTILE, SUBTILE, 0, st>>>(ps.x.p, ps.y.p, ps.z.p, ps.sbox.p);
  DS_CHECK_LAUNCH();
  const long long nb6 = (long long)ps.n_tiles * 6, ns6 = (long long)(ps.n_pad / SUBTILE) * 6;
  ps.box32.alloc(nb6);
  ps.sbox32.alloc(ns6);
  k_box_f32<<<(int)((nb6 + BLK - 1) / BLK), BLK, 0, st>>>(nb6, ps.box.p, ps.box32.p);
  DS_CHECK_LAUNCH();
  k_box_f32<<<(int)((ns6 + BLK - 1) / BLK), BLK, 0, st>>>(ns6, ps.sbox.p, ps.sbox32.p);
  DS_CHECK_LAUNCH();
  // The temporaries are freed on return in stream order (or by cudaFree,
  // which waits for the device), so the stream need not be drained here.
}

// Items per tile pair: the column sub-tiles w with (mask >> w) & 0x1111 != 0.
__global__ void k_item_count(long long n_pairs, const unsigned short* __restrict__ mask,
                             int* __restrict__ cnt) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_pairs) return;
  const unsigned m = mask[p];
  int c = 0;
#pragma unroll
  for (int w = 0; w < 4; ++w) c += ((m >> w) & 0x1111u) != 0u;
  cnt[p] = c;
}

__global__ void k_item_fill(long long n_pairs, const unsigned short* __restrict__ mask,
                            const int* __restrict__ cols, const int* __restrict__ off,
                            unsigned int* __restrict__ items) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_pairs) return;
  const unsigned m = mask[p], ct = (unsigned)cols[p];
  int o = off[p];
#pragma unroll
  for (int w = 0; w < 4; ++w) {
    const unsigned r = (m >> w) & 0x1111u;  // bit 4k: row sub-tile k
    if (r == 0u) continue;
    const unsigned rk = (r & 1u) | ((r >> 3) & 2u) | ((r >> 6) & 4u) | ((r >> 9) & 8u);
    items[o++] = (ct << 6) | ((unsigned)w << 4) | rk;
  }
}

__global__ void k_item_rows(int n_rows, const int* __restrict__ row_ptr,
                            const int* __restrict__ off, int* __restrict__ item_ptr) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t <= n_rows) item_ptr[t] = off[row_ptr[t]];
}

void build_slice_items(PairList& pl, cudaStream_t st) {
  const long long np = pl.n_pairs;
  require(np < (1ll << 29), "too many tile pairs for the item list");
  DevBuf<int> cnt, off;
  cnt.alloc(np + 1);
  off.alloc(np + 1);
  DS_CUDA(cudaMemsetAsync(cnt.p + np, 0, sizeof(int), st));
  const int g = (int)((np + BLK - 1) / BLK);
  if (np > 0) {
    k_item_count<<<g, BLK, 0, st>>>(np, pl.mask.p, cnt.p);
    DS_CHECK_LAUNCH();
  }
  size_t scan_bytes = 0;
  DS_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, cnt.p, off.p, (int)(np + 1), st));
  DevBuf<unsigned char> tmp;
  tmp.alloc(std::max<size_t>(scan_bytes, 1));
  DS_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, scan_bytes, cnt.p, off.p, (int)(np + 1), st));
  pl.items.alloc(std::max<long long>(4 * np, 1));
  if (np > 0) {
    k_item_fill<<<g, BLK, 0, st>>>(np, pl.mask.p, pl.cols.p, off.p, pl.items.p);
    DS_CHECK_LAUNCH();
  }
  pl.item_ptr.alloc(pl.n_rows + 1);
  k_item_rows<<<(pl.n_rows + 1 + BLK - 1) / BLK, BLK, 0, st>>>(pl.n_rows, pl.row_ptr.p, off.p,
                                                               pl.item_ptr.p);
  DS_CHECK_LAUNCH();
}

void build_pair_list(PairList& pl, const PointSet& rows, const PointSet& cols,
                     const KernelConsts& kc, cudaStream_t st) {
  pl.n_rows = rows.n_tiles;
  DevBuf<int> counts;  // n_rows + 1: the last one 0 for the scan's total
  counts.alloc(rows.n_tiles + 1);
  DS_CUDA(cudaMemsetAsync(counts.p + rows.n_tiles, 0, sizeof(int), st));
  const int n_groups = (cols.n_tiles + PGROUP - 1) / PGROUP;
  const CullConsts ck = cull_consts(kc);
  DevBuf<float> gbox;
  gbox.alloc((size_t)n_groups * 6);
  k_group_boxes<<<(n_groups + 127) / 128, 128, 0, st>>>(cols.n_tiles, cols.box32.p, gbox.p);
  DS_CHECK_LAUNCH();
  const size_t search_smem = (size_t)2 * n_groups * sizeof(unsigned);
  require(search_smem <= 48 * 1024, "too many column tiles for the pair search");
  k_pair_search<false><<<rows.n_tiles, BLK, search_smem, st>>>(
      rows.box32.p, cols.box32.p, gbox.p, cols.n_tiles, ck, counts.p, nullptr, nullptr);
  DS_CHECK_LAUNCH();
  // CSR offsets (exclusive scan of the counts, one trailing 0 so that
  // row_ptr[n_rows] is the total) and the launch order: rows by decreasing
  // count, ties by index (CUB's radix sort is stable), all on the device.
  const int nr = rows.n_tiles;
  pl.row_ptr.alloc(nr + 1);
  pl.row_order.alloc(nr);
  DevBuf<int> iota, keys_sorted;
  iota.alloc(nr);
  keys_sorted.alloc(nr);
  k_iota<<<(nr + BLK - 1) / BLK, BLK, 0, st>>>(nr, iota.p);
  DS_CHECK_LAUNCH();
  size_t scan_bytes = 0, sort_bytes = 0;
  DS_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, counts.p, pl.row_ptr.p, nr + 1, st));
  DS_CUDA(cub::DeviceRadixSort::SortPairsDescending(nullptr, sort_bytes, counts.p, keys_sorted.p,
                                                    iota.p, pl.row_order.p, nr, 0, 32, st));
  DevBuf<unsigned char> tmp;
  tmp.alloc(std::max<size_t>(std::max(scan_bytes, sort_bytes), 1));
  DS_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, scan_bytes, counts.p, pl.row_ptr.p, nr + 1, st));
  DS_CUDA(cub::DeviceRadixSort::SortPairsDescending(tmp.p, sort_bytes, counts.p, keys_sorted.p,
                                                    iota.p, pl.row_order.p, nr, 0, 32, st));
  int total = 0;
  DS_CUDA(cudaMemcpyAsync(&total, pl.row_ptr.p + nr, sizeof(int), cudaMemcpyDeviceToHost, st));
  DS_CUDA(cudaStreamSynchronize(st));
  require(total >= 0, "too many tile pairs");
  pl.n_pairs = total;
  pl.cols.alloc(std::max<long long>(total, 1));
  k_pair_search<true><<<rows.n_tiles, BLK, search_smem, st>>>(
      rows.box32.p, cols.box32.p, gbox.p, cols.n_tiles, ck, nullptr, pl.row_ptr.p, pl.cols.p);
  DS_CHECK_LAUNCH();
  pl.mask.alloc(std::max<long long>(total, 1));
  k_pair_mask<<<rows.n_tiles, 64, 0, st>>>(rows.n_tiles, pl.row_ptr.p, pl.cols.p, rows.sbox32.p,
                                           cols.sbox32.p, ck, pl.mask.p);
  DS_CHECK_LAUNCH();
}

}  // namespace ds
