// The learned warm start and per-skewer preconditioner (learned.cu), and the
// skewer-band preconditioner of the mixed-precision solver (skewer_pc.cu).
#pragma once

#include <cuda_bf16.h>

#include "ds_internal.cuh"

namespace ds {

constexpr int F_IN = 11;      // input features per pixel
constexpr int N_LAYERS = 4;   // message-passing layers

struct LearnedNet {
  struct Slot {
    size_t off = 0, rows = 0, cols = 0;
    bool bias = false;
  };
  ds_context* ctx;
  int H, B, NO = 0;
  KernelConsts kc;
  size_t n_params = 0;
  Slot W_in, b_in, W_l[N_LAYERS], b_l[N_LAYERS], W_o, b_o;
  DevBuf<float> params, grads, adam_m, adam_v;
  DevBuf<unsigned short> wbf;  // BF16 copy of the parameters (forward weights)
  long long step = 0;
  // per-geometry work space
  const double* rec_cur = nullptr;  // records of the last forward (device)
  size_t n_cur = 0;
  int nsk_cur = 0;
  DevBuf<int> nbr;
  DevBuf<double2> skxy;  // (x, y) per skewer
  DevBuf<float> gw, X, h[N_LAYERS + 1], Z[N_LAYERS + 1], cat[N_LAYERS], Y, dY, dh, dh2, dZ, dcat,
      part;
  DevBuf<double> dpart;
  // inference: message-passing layers on the tensor cores (learned_tc.cu)
  bool tc_infer = true;
  bool tc_active = false;
  DevBuf<float> wt;   // W^T of the layer in flight (FP32)
  DevBuf<int> tc_err;

  LearnedNet(ds_context* c, int hidden, int band, const KernelConsts& k, unsigned seed);
  void sync_weights();
  void ensure(int n_sk, int n_per);
  void gemm_fwd(int M, int N, int K, const float* A, int lda, const Slot& W, const Slot& b,
                float* Zp, float* out, const float* res, int epi);
  void grad_w(int M, int K, int N, const float* A, int lda, const float* D, const Slot& W,
              const Slot& b);
  // records: W-form records (x, y, z, w, w d) of n_sk skewers x n_per pixels,
  // skewer-contiguous, on the device
  void forward(int n_sk, int n_per, const double* rec);
  void outputs(int n_sk, int n_per, double* y0, float* Lrows);
  void loss_and_grad(int n_sk, int n_per, const double* rec, const double* ystar,
                     const float* probe, float wx, float wp, double* losses);
  void backward(int n_sk, int n_per);
  void adam_step(float lr);
};

// Band preconditioner M^-1 = L L^T of an operator over blocks of `n_per`
// slots (FP32 L rows of bandwidth `band`, indexed by slot): per skewer (slot
// = record, blocks of n_per consecutive records) or per cluster of
// neighbouring skewers (crec: the record of each slot, -1 on padding).
bool layer_tc_usable(int M, int N, int K);
void launch_layer_tc(int M, const float* A, const __nv_bfloat16* W, const float* bias, float* Z,
                     float* out, const float* res, float* wt, int* err, cudaStream_t st);

struct SkewerPC {
  int n_sk = 0, n_per = 0, band = 0;  // blocks, slots per block, bandwidth
  DevBuf<float> L;    // band + 1 planes of n_sk n_per slots: L[k][k - m] at plane m
  DevBuf<int> crec;   // record of each slot (empty: slot = record)
  int n_fallback = 0;  // cluster factor: columns that fell back to Jacobi
  // skewers per block and the skewers of each block (g per block, -1 on
  // padding; empty: block b is skewer b, g = 1)
  int g = 1;
  DevBuf<int> bsk;
};

}  // namespace ds

struct ds_learned {
  std::unique_ptr<ds::LearnedNet> net;
};
