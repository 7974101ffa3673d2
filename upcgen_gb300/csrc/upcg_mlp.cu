// Learned surrogate of the realistic photon flux.
//
// An MLP maps u = normalised (ln w, ln b, R, a, ln g) to
//   y = ln( Q_ff(w, b) / Q_pt(w, b) ),
// the log-ratio of the Woods-Saxon form-factor flux amplitude of fluxForm
// (src/UpcCrossSection.cpp:181-218; F normalised to F(0) = 1, clamp at
// Q2max - dQ2 as :188) to the point-charge amplitude Q_pt = k K1(k b / hc),
// k = w / g.  The flux follows as N = factor (Q_pt e^y)^2 / w.  Five inputs,
// four hidden layers of 128 SiLU units, one output; BF16 weights in the
// products, FP32 accumulation, FP32 master weights and Adam state.
//
// Kernels: k_mlp_labels (training points and quadrature labels),
// k_mlp_step (fused forward + backward over a batch, per-CTA gradient
// partials, no atomics), k_mlp_adam (fixed-order reduction of the partials and
// the Adam update), k_mlp_infer (forward only).
#include <cuda_bf16.h>

#include "upcg_device.cuh"
#include "upcg_internal.h"

namespace upcg {

namespace {

constexpr int kIn = 5, kH = 128;
constexpr int kWs = kH + 2;  // padded row stride of a weight matrix in shared memory (bf16)
// parameter offsets (FP32 master vector)
constexpr int oW1 = 0, oB1 = oW1 + kH * kIn;
constexpr int oW2 = oB1 + kH, oB2 = oW2 + kH * kH;
constexpr int oW3 = oB2 + kH, oB3 = oW3 + kH * kH;
constexpr int oW4 = oB3 + kH, oB4 = oW4 + kH * kH;
constexpr int oW5 = oB4 + kH, oB5 = oW5 + kH;
constexpr int kParams = oB5 + 1;
constexpr int kStepSamples = 32;   // samples per CTA of k_mlp_step
constexpr int kStepThreads = 256;

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float silu_d(float z) {
  const float s = 1.f / (1.f + __expf(-z));
  return s * (1.f + z * (1.f - s));
}

// counter-based uniform in [0, 1) (splitmix64 of seed, index, stream)
__device__ __forceinline__ double urand(uint64_t seed, uint64_t i, uint32_t stream) {
  uint64_t x = seed ^ (i * 0x9E3779B97F4A7C15ull) ^ ((uint64_t)stream << 56);
  x ^= x >> 30;
  x *= 0xBF58476D1CE4E5B9ull;
  x ^= x >> 27;
  x *= 0x94D049BB133111EBull;
  x ^= x >> 31;
  return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

// calcFormFac (src/UpcCrossSection.cpp:436-445) / A, FP32: rho_hat = rho0 / A
__device__ float formfac_hat(float q2, float R, float a, float rho_hat) {
  const float pi = 3.14159265358979f;
  const float Q = sqrtf(q2) / (float)kHc;
  const float x = pi * Q * a;
  const float ch = coshf(x), sh = sinhf(x);
  float sn, cs;
  sincosf(Q * R, &sn, &cs);
  float ff = 4.f * pi * pi * rho_hat * a * a * a / (Q * a * Q * a * sh * sh) *
             (x * ch * sn - Q * R * cs * sh);
  ff += 8.f * pi * rho_hat * a * a * a * expf(-R / a) / ((1.f + Q * Q * a * a) * (1.f + Q * Q * a * a));
  return ff;
}

// rho0 / A of calcWSRho (:152-163): 200-node Simpson over [0, 20] fm
__device__ float ws_rho_hat(float R, float a) {
  const int nb = 200;
  const float db = 20.f / (nb - 1);
  float s = 0.f;
  for (int i = 0; i < nb; ++i) {
    const float r = i * db;
    const float v = r * r / (1.f + expf((r - R) / a));
    s += v * ((i == 0 || i == nb - 1) ? 1.f : ((i & 1) ? 4.f : 2.f));
  }
  return 1.f / (s * db / 3.f) / 4.f / 3.14159265358979f;
}


__device__ __forceinline__ void normalise(const MlpBox& bx, float lw, float lb, float R, float a,
                                          float lg, float* u) {
  u[0] = 2.f * (lw - bx.lw_lo) / (bx.lw_hi - bx.lw_lo) - 1.f;
  u[1] = 2.f * (lb - logf(bx.bf_lo * bx.R_lo)) / (bx.lb_hi - logf(bx.bf_lo * bx.R_lo)) - 1.f;
  u[2] = 2.f * (R - bx.R_lo) / (bx.R_hi - bx.R_lo) - 1.f;
  u[3] = 2.f * (a - bx.a_lo) / (bx.a_hi - bx.a_lo) - 1.f;
  u[4] = 2.f * (lg - logf(bx.g_lo)) / (logf(bx.g_hi) - logf(bx.g_lo)) - 1.f;
}

// Training points, uniform in R, a, g and log-uniform in w and b (b from
// bf_lo R to b_hi), with their labels.  Labels: for b <= 2R the q-integral
// of fluxForm by composite Gauss-Legendre (128 panels x 12 nodes on [0, 10]
// GeV; integrand in FP32, sum in FP64); beyond 2R, where the charge lies
// inside b, the amplitude is Q_pt times Phi(k) = int rho sinh(k r)/(k r) /
// int rho (Simpson, 400 nodes).  Points with k b / hc > 30 (flux below
// e^-60 of its scale) get weight 0.
__global__ void k_mlp_labels(MlpBox bx, uint64_t seed, uint64_t i0, int n, const double* glx,
                             const double* glw, float* __restrict__ xs, float* __restrict__ ys,
                             float* __restrict__ ws) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const uint64_t id = i0 + (uint64_t)t;
  const float R = bx.R_lo + (bx.R_hi - bx.R_lo) * (float)urand(seed, id, 0);
  const float a = bx.a_lo + (bx.a_hi - bx.a_lo) * (float)urand(seed, id, 1);
  const float g = bx.g_lo + (bx.g_hi - bx.g_lo) * (float)urand(seed, id, 2);
  const float lw = bx.lw_lo + (bx.lw_hi - bx.lw_lo) * (float)urand(seed, id, 3);
  const float lb0 = logf(bx.bf_lo * R);
  const float lb = lb0 + (bx.lb_hi - lb0) * (float)urand(seed, id, 4);
  float u[kIn];
  normalise(bx, lw, lb, R, a, logf(g), u);
  for (int j = 0; j < kIn; ++j) xs[(size_t)t * kIn + j] = u[j];
  const float w = expf(lw), b = expf(lb);
  const float k = w / g;                // GeV
  const float kf = k / (float)kHc;      // fm^-1
  const float xpt = kf * b;
  if (xpt > 30.f) {
    ys[t] = 0.f;
    ws[t] = 0.f;
    return;
  }
  double K0, K1;
  bessel_k01((double)xpt, K0, K1);
  const double qpt = (double)k * K1;
  const float rho_hat = ws_rho_hat(R, a);
  double q;
  if (b <= 2.f * R) {
    const float q2max = 2.f, q2clamp = 2.f - (2.f - 1e-9f) / 1e6f;
    const float k2 = k * k;
    double s = 0.;
    for (int pa = 0; pa < 128; ++pa) {
      const float lo = 10.f * pa / 128.f, hw = 0.5f * 10.f / 128.f;
      float ps = 0.f;
      for (int j = 0; j < 12; ++j) {
        const float qq = lo + hw * (1.f + (float)glx[j]);
        const float tq = qq * qq + k2;
        const float f = formfac_hat(tq < q2max ? tq : q2clamp, R, a, rho_hat);
        ps += (float)glw[j] * hw * (qq * qq * f / tq) * j1f(b * qq / (float)kHc);
      }
      s += (double)ps;
    }
    q = s;
  } else {
    const int nr = 400;
    const float dr = 20.f / nr;
    double num = 0., den = 0.;
    for (int i = 0; i <= nr; ++i) {
      const float r = i * dr;
      const float wt = (i == 0 || i == nr) ? 1.f : ((i & 1) ? 4.f : 2.f);
      const float rho = 1.f / (1.f + expf((r - R) / a));
      const float kr = kf * r;
      const float shk = kr > 1e-4f ? sinhf(kr) / kr : 1.f + kr * kr / 6.f;
      num += (double)(wt * r * r * rho * shk);
      den += (double)(wt * r * r * rho);
    }
    q = qpt * num / den;
  }
  const bool ok = q > 0. && qpt > 0.;
  ys[t] = ok ? (float)log(q / qpt) : 0.f;
  ws[t] = ok ? 1.f : 0.f;
}

// Shared-memory image of the network for one CTA: bf16 weights with padded
// rows (conflict-free both for output-major and input-major walks).
struct MlpSmem {
  __nv_bfloat16 w1[kH][kIn];
  __nv_bfloat16 w[3][kH][kWs];  // W2..W4 [out][in]
  float w5[kH];
  float b[4][kH];
  float b5;
};

__device__ void load_net(MlpSmem& S, const __nv_bfloat16* __restrict__ pb, const float* __restrict__ pf) {
  for (int i = threadIdx.x; i < kH * kIn; i += blockDim.x) S.w1[i / kIn][i % kIn] = pb[oW1 + i];
  for (int l = 0; l < 3; ++l) {
    const int off = l == 0 ? oW2 : (l == 1 ? oW3 : oW4);
    for (int i = threadIdx.x; i < kH * kH; i += blockDim.x) S.w[l][i / kH][i % kH] = pb[off + i];
  }
  for (int i = threadIdx.x; i < kH; i += blockDim.x) {
    S.w5[i] = __bfloat162float(pb[oW5 + i]);
    S.b[0][i] = pf[oB1 + i];
    S.b[1][i] = pf[oB2 + i];
    S.b[2][i] = pf[oB3 + i];
    S.b[3][i] = pf[oB4 + i];
  }
  if (threadIdx.x == 0) S.b5 = pf[oB5];
}

// forward of ns samples: z[l][s][o] pre-activations (l = 0..3), y[s]
// act[s][i] = SiLU(z[s][i]), once per layer (not once per output neuron)
template <int NS>
__device__ __forceinline__ void activate(const float (*z)[kH], float (*act)[kH]) {
  for (int e = threadIdx.x; e < NS * kH; e += blockDim.x) act[e / kH][e % kH] = silu(z[e / kH][e % kH]);
}

template <int NS>
__device__ void forward(const MlpSmem& S, const float (*u)[kIn], float (*z)[NS][kH],
                        float (*act)[kH], float* y) {
  const int o = threadIdx.x & (kH - 1), sg = threadIdx.x >> 7;  // 2 sample groups
  constexpr int per = NS / 2;
  {
    float acc[per];
#pragma unroll
    for (int k = 0; k < per; ++k) {
      const int s = sg + 2 * k;
      float v = S.b[0][o];
#pragma unroll
      for (int i = 0; i < kIn; ++i) v += __bfloat162float(S.w1[o][i]) * u[s][i];
      acc[k] = v;
    }
#pragma unroll
    for (int k = 0; k < per; ++k) z[0][sg + 2 * k][o] = acc[k];
  }
  __syncthreads();
  for (int l = 1; l < 4; ++l) {
    activate<NS>(z[l - 1], act);
    __syncthreads();
    float acc[per];
#pragma unroll
    for (int k = 0; k < per; ++k) acc[k] = S.b[l][o];
    for (int i = 0; i < kH; ++i) {
      const float wv = __bfloat162float(S.w[l - 1][o][i]);
#pragma unroll
      for (int k = 0; k < per; ++k) acc[k] += wv * act[sg + 2 * k][i];
    }
    __syncthreads();  // act is rewritten by the next layer
#pragma unroll
    for (int k = 0; k < per; ++k) z[l][sg + 2 * k][o] = acc[k];
    __syncthreads();
  }
  activate<NS>(z[3], act);
  __syncthreads();
  // output: one warp per sample group of samples, lanes over neurons
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int s = wid; s < NS; s += blockDim.x / 32) {
    float v = 0.f;
    for (int i = lane; i < kH; i += 32) v += S.w5[i] * act[s][i];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (lane == 0) y[s] = v + S.b5;
  }
  __syncthreads();
}

// One CTA: kStepSamples samples; writes this CTA's gradient of
// sum_s w_s (y_s - t_s)^2 / wsum into part[cta][kParams]; loss into lossp[cta].
__global__ void __launch_bounds__(kStepThreads) k_mlp_step(
    const __nv_bfloat16* __restrict__ pb, const float* __restrict__ pf, const float* __restrict__ xs,
    const float* __restrict__ ys, const float* __restrict__ ws, const int* __restrict__ idx,
    int nbatch, float inv_wsum, float* __restrict__ part, float* __restrict__ lossp) {
  constexpr int NS = kStepSamples;
  extern __shared__ __align__(16) uint8_t smem[];
  MlpSmem& S = *reinterpret_cast<MlpSmem*>(smem);
  float(*z)[NS][kH] = reinterpret_cast<float(*)[NS][kH]>(smem + sizeof(MlpSmem));
  float(*d)[kH] = reinterpret_cast<float(*)[kH]>(smem + sizeof(MlpSmem) + sizeof(float) * 4 * NS * kH);
  float(*dn)[kH] = d + NS;
  float(*act)[kH] = dn + NS;
  __shared__ float u[NS][kIn], y[NS], g[NS];
  load_net(S, pb, pf);
  const int base = blockIdx.x * NS;
  for (int e = threadIdx.x; e < NS * kIn; e += blockDim.x) {
    const int s = e / kIn, j = e % kIn;
    u[s][j] = base + s < nbatch ? xs[(size_t)idx[base + s] * kIn + j] : 0.f;
  }
  __syncthreads();
  forward<NS>(S, u, z, act, y);
  float* P = part + (size_t)blockIdx.x * kParams;
  if (threadIdx.x < NS) {
    const int s = threadIdx.x;
    float gv = 0.f, lv = 0.f;
    if (base + s < nbatch) {
      const int id = idx[base + s];
      const float r = y[s] - ys[id];
      gv = 2.f * ws[id] * r * inv_wsum;
      lv = ws[id] * r * r * inv_wsum;
    }
    g[s] = gv;
    y[s] = lv;  // reuse: per-sample loss
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float l = 0.f;
    for (int s = 0; s < NS; ++s) l += y[s];
    lossp[blockIdx.x] = l;
  }
  const int o = threadIdx.x & (kH - 1), sg = threadIdx.x >> 7;
  // output layer: dW5[i] = sum_s g_s a4[s][i], db5 = sum_s g_s; delta4 = g W5 silu'(z4)
  // (act holds a4 after the forward pass)
  if (threadIdx.x < kH) {
    float acc = 0.f;
    for (int s = 0; s < NS; ++s) acc += g[s] * act[s][o];
    P[oW5 + o] = acc;
  }
  if (threadIdx.x == kH) {
    float acc = 0.f;
    for (int s = 0; s < NS; ++s) acc += g[s];
    P[oB5] = acc;
  }
  for (int s = sg; s < NS; s += 2) d[s][o] = g[s] * S.w5[o] * silu_d(z[3][s][o]);
  __syncthreads();
  // hidden layers 4 .. 2: weights of layer l (W[l-1] in S.w) map a_{l-1} -> z_l
  for (int l = 3; l >= 1; --l) {
    const int offW = l == 1 ? oW2 : (l == 2 ? oW3 : oW4);
    const int offB = l == 1 ? oB2 : (l == 2 ? oB3 : oB4);
    // dW[o][i] = sum_s d[s][o] a_{l-1}[s][i]; each thread 64 entries
    activate<NS>(z[l - 1], act);
    __syncthreads();
    for (int e = threadIdx.x; e < kH * kH; e += blockDim.x) {
      const int oo = e / kH, ii = e % kH;
      float acc = 0.f;
#pragma unroll 4
      for (int s = 0; s < NS; ++s) acc += d[s][oo] * act[s][ii];
      P[offW + e] = acc;
    }
    if (threadIdx.x < kH) {
      float acc = 0.f;
      for (int s = 0; s < NS; ++s) acc += d[s][threadIdx.x];
      P[offB + threadIdx.x] = acc;
    }
    // delta_{l-1}[s][i] = (sum_o W[o][i] d[s][o]) silu'(z_{l-1}[s][i]), i = o here
    {
      const int i = o;
      for (int s = sg; s < NS; s += 2) {
        float acc = 0.f;
        for (int oo = 0; oo < kH; ++oo) acc += __bfloat162float(S.w[l - 1][oo][i]) * d[s][oo];
        dn[s][i] = acc * silu_d(z[l - 1][s][i]);
      }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < NS * kH; e += blockDim.x) d[e / kH][e % kH] = dn[e / kH][e % kH];
    __syncthreads();
  }
  // first layer: dW1[o][j] = sum_s d[s][o] u[s][j], db1
  for (int e = threadIdx.x; e < kH * kIn; e += blockDim.x) {
    const int oo = e / kIn, j = e % kIn;
    float acc = 0.f;
    for (int s = 0; s < NS; ++s) acc += d[s][oo] * u[s][j];
    P[oW1 + e] = acc;
  }
  if (threadIdx.x < kH) {
    float acc = 0.f;
    for (int s = 0; s < NS; ++s) acc += d[s][threadIdx.x];
    P[oB1 + threadIdx.x] = acc;
  }
}

// gradient = sum of the CTA partials in CTA order; Adam (Kingma & Ba 2015)
__global__ void k_mlp_adam(const float* __restrict__ part, int nparts, float* __restrict__ pf,
                           __nv_bfloat16* __restrict__ pb, float* __restrict__ m,
                           float* __restrict__ v, float lr, float b1, float b2, float eps,
                           float bc1, float bc2, float* __restrict__ grad_out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  float gsum = 0.f;
  for (int c = 0; c < nparts; ++c) gsum += part[(size_t)c * kParams + i];
  if (grad_out) {
    grad_out[i] = gsum;
    return;
  }
  const float mi = b1 * m[i] + (1.f - b1) * gsum;
  const float vi = b2 * v[i] + (1.f - b2) * gsum * gsum;
  m[i] = mi;
  v[i] = vi;
  const float p = pf[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  pf[i] = p;
  pb[i] = __float2bfloat16(p);
}

__global__ void k_mlp_to_bf16(const float* __restrict__ pf, __nv_bfloat16* __restrict__ pb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kParams) pb[i] = __float2bfloat16(pf[i]);
}

constexpr int kInferSamples = 64;
constexpr int kAs = kH + 8;  // padded row stride (bf16) of the tensor-core operands

// Inference on the tensor cores (mma.sync m16n8k16, bf16 in, FP32 accumulate):
// per 64-sample tile and layer, act[64][128] . W^T; activations between
// layers rounded to bf16 (the operand type), bias + SiLU in FP32.
struct MlpSmemI {
  __nv_bfloat16 w1[kH][kIn];
  __align__(16) __nv_bfloat16 w[3][kH][kAs];  // [l][out][in]
  __align__(16) __nv_bfloat16 act[2][kInferSamples][kAs];
  float w5[kH];
  float b[4][kH];
  float b5;
};

__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
      "{%8, %9}, {%0, %1, %2, %3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__global__ void __launch_bounds__(kStepThreads) k_mlp_infer(const __nv_bfloat16* __restrict__ pb,
                                                            const float* __restrict__ pf,
                                                            const float* __restrict__ xs, int n,
                                                            float* __restrict__ out) {
  constexpr int NS = kInferSamples;
  extern __shared__ __align__(16) uint8_t smem[];
  MlpSmemI& S = *reinterpret_cast<MlpSmemI*>(smem);
  __shared__ float u[NS][kIn], y[NS];
  for (int i = threadIdx.x; i < kH * kIn; i += blockDim.x) S.w1[i / kIn][i % kIn] = pb[oW1 + i];
  // hidden weights: 16-byte loads (the offsets are multiples of 8 bf16)
  static_assert(oW2 % 8 == 0 && oW3 % 8 == 0 && oW4 % 8 == 0 && (kAs * 2) % 16 == 0, "alignment");
  for (int l = 0; l < 3; ++l) {
    const int off = l == 0 ? oW2 : (l == 1 ? oW3 : oW4);
    const uint4* src = reinterpret_cast<const uint4*>(pb + off);
    for (int i = threadIdx.x; i < kH * (kH / 8); i += blockDim.x)
      *reinterpret_cast<uint4*>(&S.w[l][i / (kH / 8)][(i % (kH / 8)) * 8]) = __ldg(src + i);
  }
  for (int i = threadIdx.x; i < kH; i += blockDim.x) {
    S.w5[i] = __bfloat162float(pb[oW5 + i]);
    S.b[0][i] = pf[oB1 + i];
    S.b[1][i] = pf[oB2 + i];
    S.b[2][i] = pf[oB3 + i];
    S.b[3][i] = pf[oB4 + i];
  }
  if (threadIdx.x == 0) S.b5 = pf[oB5];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // warp w: rows 16 (w & 3) .. +16, output columns 64 (w >> 2) .. +64 (8 n-blocks)
  const int m0 = 16 * (warp & 3), n0 = 64 * (warp >> 2);
  const int r = lane >> 2, c = (lane & 3) * 2;
  const int ntiles = (n + NS - 1) / NS;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int base = tile * NS;
    for (int e = threadIdx.x; e < NS * kIn; e += blockDim.x) {
      const int s = e / kIn, j = e % kIn;
      u[s][j] = base + s < n ? xs[(size_t)(base + s) * kIn + j] : 0.f;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < NS * kH; e += blockDim.x) {  // layer 1 (5 inputs)
      const int s = e / kH, o = e % kH;
      float v = S.b[0][o];
#pragma unroll
      for (int j = 0; j < kIn; ++j) v += __bfloat162float(S.w1[o][j]) * u[s][j];
      S.act[0][s][o] = __float2bfloat16(silu(v));
    }
    __syncthreads();
    int cur = 0;
    for (int l = 0; l < 3; ++l) {
      float d[8][4];
#pragma unroll
      for (int nb = 0; nb < 8; ++nb)
#pragma unroll
        for (int q = 0; q < 4; ++q) d[nb][q] = 0.f;
#pragma unroll
      for (int k0 = 0; k0 < kH; k0 += 16) {
        uint32_t af[4];
        af[0] = *reinterpret_cast<const uint32_t*>(&S.act[cur][m0 + r][k0 + c]);
        af[1] = *reinterpret_cast<const uint32_t*>(&S.act[cur][m0 + r + 8][k0 + c]);
        af[2] = *reinterpret_cast<const uint32_t*>(&S.act[cur][m0 + r][k0 + c + 8]);
        af[3] = *reinterpret_cast<const uint32_t*>(&S.act[cur][m0 + r + 8][k0 + c + 8]);
#pragma unroll
        for (int nb = 0; nb < 8; ++nb) {
          const int nn = n0 + 8 * nb + r;  // output neuron of this lane's B column
          uint32_t bf[2];
          bf[0] = *reinterpret_cast<const uint32_t*>(&S.w[l][nn][k0 + c]);
          bf[1] = *reinterpret_cast<const uint32_t*>(&S.w[l][nn][k0 + c + 8]);
          mma16816(d[nb], af, bf);
        }
      }
      // bias + SiLU -> the other activation buffer (bf16)
#pragma unroll
      for (int nb = 0; nb < 8; ++nb) {
        const int col = n0 + 8 * nb + c;
        const float b0 = S.b[l + 1][col], b1 = S.b[l + 1][col + 1];
        *reinterpret_cast<__nv_bfloat162*>(&S.act[cur ^ 1][m0 + r][col]) =
            __floats2bfloat162_rn(silu(d[nb][0] + b0), silu(d[nb][1] + b1));
        *reinterpret_cast<__nv_bfloat162*>(&S.act[cur ^ 1][m0 + r + 8][col]) =
            __floats2bfloat162_rn(silu(d[nb][2] + b0), silu(d[nb][3] + b1));
      }
      cur ^= 1;
      __syncthreads();
    }
    for (int s = warp; s < NS; s += blockDim.x / 32) {
      float v = 0.f;
      for (int i = lane; i < kH; i += 32) v += S.w5[i] * __bfloat162float(S.act[cur][s][i]);
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
      if (lane == 0) y[s] = v + S.b5;
    }
    __syncthreads();
    if (threadIdx.x < NS && base + (int)threadIdx.x < n) out[base + threadIdx.x] = y[threadIdx.x];
  }
}

__global__ void k_mlp_table_inputs(MlpBox bx, FastFluxTables t, int w0, int w1, float R, float a,
                                   float lg, float* __restrict__ xs) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (w1 - w0) * t.nb) return;
  const int iw = w0 + e / t.nb, j = e % t.nb;
  float u[kIn];
  normalise(bx, (float)(t.lw0 + iw * t.hw), (float)(t.lb0 + j * t.hb), R, a, lg, u);
  for (int q = 0; q < kIn; ++q) xs[(size_t)e * kIn + q] = u[q];
}

// Q table entries A Q_pt e^y (the table holds the un-normalised amplitude)
__global__ void k_mlp_table_fill(FastFluxTables t, int w0, int w1, double g, double A,
                                 const float* __restrict__ ys) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (w1 - w0) * t.nb) return;
  const int iw = w0 + e / t.nb, j = e % t.nb;
  const double k = exp(t.lw0 + iw * t.hw) / g;
  const double b = exp(t.lb0 + j * t.hb);
  double K0, K1;
  bessel_k01(k * b / kHc, K0, K1);
  const double q = A * k * K1 * exp((double)ys[e]);
  t.qt[(size_t)iw * t.nb + j] = q;
  t.qt32[(size_t)iw * t.nb + j] = (float)q;
}

}  // namespace

cudaError_t launch_mlp_table_inputs(const MlpBox& bx, const FastFluxTables& t, int w0, int w1,
                                    float R, float a, float g, float* xs, cudaStream_t st) {
  const int n = (w1 - w0) * t.nb;
  if (n <= 0) return cudaSuccess;
  note_launch();
  k_mlp_table_inputs<<<(n + 255) / 256, 256, 0, st>>>(bx, t, w0, w1, R, a, logf(g), xs);
  return cudaGetLastError();
}

cudaError_t launch_mlp_table_fill(const FastFluxTables& t, int w0, int w1, double g, double A,
                                  const float* ys, cudaStream_t st) {
  const int n = (w1 - w0) * t.nb;
  if (n <= 0) return cudaSuccess;
  note_launch();
  k_mlp_table_fill<<<(n + 255) / 256, 256, 0, st>>>(t, w0, w1, g, A, ys);
  return cudaGetLastError();
}

int mlp_param_count() { return kParams; }

size_t mlp_step_smem() { return sizeof(MlpSmem) + sizeof(float) * (4 + 3) * kStepSamples * kH; }
size_t mlp_infer_smem() { return sizeof(MlpSmemI); }
int mlp_step_samples() { return kStepSamples; }

cudaError_t launch_mlp_labels(const MlpBox& bx, uint64_t seed, uint64_t i0, int n,
                              const double* d_glx, const double* d_glw, float* xs, float* ys,
                              float* ws, cudaStream_t st) {
  note_launch();
  k_mlp_labels<<<(n + 127) / 128, 128, 0, st>>>(bx, seed, i0, n, d_glx, d_glw, xs, ys, ws);
  return cudaGetLastError();
}

cudaError_t launch_mlp_step(const void* pb, const float* pf, const float* xs, const float* ys,
                            const float* ws, const int* idx, int nbatch, float inv_wsum,
                            float* part, float* lossp, cudaStream_t st) {
  static std::atomic<uint64_t> attr{0};  // devices with the limit raised
  {
    const cudaError_t ea = smem_attr_once(attr, k_mlp_step, (int)mlp_step_smem());
    if (ea != cudaSuccess) return ea;
  }
  const int ctas = (nbatch + kStepSamples - 1) / kStepSamples;
  note_launch();
  k_mlp_step<<<ctas, kStepThreads, mlp_step_smem(), st>>>(
      static_cast<const __nv_bfloat16*>(pb), pf, xs, ys, ws, idx, nbatch, inv_wsum, part, lossp);
  return cudaGetLastError();
}

cudaError_t launch_mlp_adam(const float* part, int nparts, float* pf, void* pb, float* m, float* v,
                            float lr, int step, float* grad_out, cudaStream_t st) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float bc1 = 1.f - powf(b1, (float)step), bc2 = 1.f - powf(b2, (float)step);
  note_launch();
  k_mlp_adam<<<(kParams + 255) / 256, 256, 0, st>>>(part, nparts, pf,
                                                     static_cast<__nv_bfloat16*>(pb), m, v, lr, b1,
                                                     b2, eps, bc1, bc2, grad_out);
  return cudaGetLastError();
}

cudaError_t launch_mlp_to_bf16(const float* pf, void* pb, cudaStream_t st) {
  note_launch();
  k_mlp_to_bf16<<<(kParams + 255) / 256, 256, 0, st>>>(pf, static_cast<__nv_bfloat16*>(pb));
  return cudaGetLastError();
}

cudaError_t launch_mlp_infer(const void* pb, const float* pf, const float* xs, int n, float* out,
                             cudaStream_t st) {
  static std::atomic<uint64_t> attr{0};  // devices with the limit raised
  {
    const cudaError_t ea = smem_attr_once(attr, k_mlp_infer, (int)mlp_infer_smem());
    if (ea != cudaSuccess) return ea;
  }
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int tiles = (n + kInferSamples - 1) / kInferSamples;
  note_launch();
  k_mlp_infer<<<tiles < sms ? tiles : sms, kStepThreads, mlp_infer_smem(), st>>>(
      static_cast<const __nv_bfloat16*>(pb), pf, xs, n, out);
  return cudaGetLastError();
}

}  // namespace upcg
