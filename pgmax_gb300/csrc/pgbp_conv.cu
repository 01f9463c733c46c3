// Kernels of the warm-start network: 3x3 convolutions with circular padding over NHWC BF16
// images on the tensor cores (mma.sync m16n8k16 BF16, FP32 accumulation), their input and weight
// gradients, a mean-centred squared-error loss and Adam. The network (pgmax_gb300/warmstart)
// predicts BP's initial log-messages on a toroidal grid, hence the circular padding.
//
// Layouts: images [n][h][w][c] BF16 (c contiguous); weights [9][co][ci] BF16 with tap
// t = (dy + 1) * 3 + (dx + 1): out[p][o] = bias[o] + sum_t sum_i in[p + (dy, dx)][i] * w[t][o][i]
// (coordinates modulo h and w). The input gradient is the same convolution of the output
// gradient with w'[t][i][o] = w[8 - t][o][i] (pgbp_conv3x3_flip).
#include <cuda_bf16.h>
#include <stdint.h>

#include <algorithm>

#include "../../include/pgbp_learn.h"
#include "pgbp_internal.h"

namespace {

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4],
                                         const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p) {
  return *reinterpret_cast<const uint32_t*>(p);
}

// ------------------------------------------------------------------------------- forward
// One CTA step = kRows consecutive output rows of one image (fewer at the image's last rows);
// w % 16 == 0, w <= 128. Warp m owns row m / (w / 16) of the step and pixels 16 (m % (w / 16)) ..
// + 15, all co output channels. Weights stay in shared memory for the CTA's whole range of steps;
// the kRows + 2 input rows a step reads are staged once per step (each serves three output rows),
// with 16-byte copies.
template <int CI, int CO>
struct ConvSmem {
  static constexpr int kLd = CI + 8;  // BF16 row stride (conflict-free 32-bit fragment loads)
  static constexpr int kRows = 4;     // output rows per CTA step
  static size_t bytes(int w) {
    return sizeof(__nv_bfloat16) * (size_t)(9 * CO + (kRows + 2) * w) * kLd;
  }
};

template <int CI, int CO>
__global__ void __launch_bounds__(1024) conv3x3_kernel(int64_t n, int h, int w,
                                                       const __nv_bfloat16* __restrict__ in,
                               const __nv_bfloat16* __restrict__ wts,
                               const float* __restrict__ bias, void* __restrict__ out,
                               int out_f32, int relu, const __nv_bfloat16* __restrict__ mask,
                               int64_t steps_per_cta) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int kLd = ConvSmem<CI, CO>::kLd;
  constexpr int kRows = ConvSmem<CI, CO>::kRows;
  __nv_bfloat16* s_w = reinterpret_cast<__nv_bfloat16*>(smem_raw);  // [9][CO][kLd]
  __nv_bfloat16* s_in = s_w + 9 * CO * kLd;                          // [kRows + 2][w][kLd]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gid = lane >> 2, tig = lane & 3;
  const int wpr = w / 16;             // warps per output row
  const int j = warp / wpr;           // this warp's row within a step
  const int x0 = (warp % wpr) * 16;   // and its first pixel
  for (int x = threadIdx.x; x < 9 * CO * CI; x += blockDim.x) {
    const int t = x / (CO * CI), o = (x / CI) % CO, i = x % CI;
    s_w[(t * CO + o) * kLd + i] = wts[x];
  }
  const int64_t per_image = (h + kRows - 1) / kRows;
  const int64_t total = n * per_image;
  const int64_t g0 = (int64_t)blockIdx.x * steps_per_cta;
  const int64_t g1 = g0 + steps_per_cta < total ? g0 + steps_per_cta : total;
  for (int64_t g = g0; g < g1; ++g) {
    const int64_t b = g / per_image;
    const int y0 = (int)(g % per_image) * kRows;
    const int nrows = h - y0 < kRows ? h - y0 : kRows;
    __syncthreads();  // previous step's fragments read (and the weights stored)
    // input rows y0 - 1 .. y0 + nrows (circular), 8 channels per copy
    for (int x = threadIdx.x; x < (nrows + 2) * w * (CI / 8); x += blockDim.x) {
      const int dy = x / (w * (CI / 8)), px = (x / (CI / 8)) % w, i8 = x % (CI / 8);
      const int yy = (y0 + dy - 1 + h) % h;
      *reinterpret_cast<uint4*>(s_in + (dy * w + px) * kLd + 8 * i8) =
          *reinterpret_cast<const uint4*>(in + ((b * h + yy) * w + px) * CI + 8 * i8);
    }
    __syncthreads();
    if (j < nrows) {
      const int y = y0 + j;
      float acc[CO / 8][4];
#pragma unroll
      for (int nb = 0; nb < CO / 8; ++nb)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[nb][e] = 0.0f;
#pragma unroll
      for (int t = 0; t < 9; ++t) {
        const int dy = t / 3, dx = t % 3 - 1;
        const int xa = (x0 + gid + dx + w) % w, xb = (x0 + gid + 8 + dx + w) % w;
        const __nv_bfloat16* ra = s_in + ((j + dy) * w + xa) * kLd;
        const __nv_bfloat16* rb = s_in + ((j + dy) * w + xb) * kLd;
#pragma unroll
        for (int k0 = 0; k0 < CI; k0 += 16) {
          const uint32_t a[4] = {ld32(ra + k0 + 2 * tig), ld32(rb + k0 + 2 * tig),
                                 ld32(ra + k0 + 2 * tig + 8), ld32(rb + k0 + 2 * tig + 8)};
#pragma unroll
          for (int nb = 0; nb < CO / 8; ++nb) {
            const __nv_bfloat16* wr = s_w + (t * CO + nb * 8 + gid) * kLd + k0 + 2 * tig;
            const uint32_t bb[2] = {ld32(wr), ld32(wr + 8)};
            mma_bf16(acc[nb], a, bb);
          }
        }
      }
      // epilogue: bias, ReLU, mask, store (two consecutive channels per register pair)
#pragma unroll
      for (int nb = 0; nb < CO / 8; ++nb) {
        const int o = nb * 8 + 2 * tig;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          const int px = x0 + gid + 8 * half;
          const int64_t p = (b * h + y) * w + px;
          float v0 = acc[nb][2 * half] + (bias ? bias[o] : 0.0f);
          float v1 = acc[nb][2 * half + 1] + (bias ? bias[o + 1] : 0.0f);
          if (relu) {
            v0 = fmaxf(v0, 0.0f);
            v1 = fmaxf(v1, 0.0f);
          }
          if (mask) {
            if (!(__bfloat162float(mask[p * CO + o]) > 0.0f)) v0 = 0.0f;
            if (!(__bfloat162float(mask[p * CO + o + 1]) > 0.0f)) v1 = 0.0f;
          }
          if (out_f32) {
            float2* dst = reinterpret_cast<float2*>(static_cast<float*>(out) + p * CO + o);
            *dst = make_float2(v0, v1);
          } else {
            __nv_bfloat162* dst = reinterpret_cast<__nv_bfloat162*>(
                static_cast<__nv_bfloat16*>(out) + p * CO + o);
            *dst = __floats2bfloat162_rn(v0, v1);
          }
        }
      }
    }
  }
}

// ------------------------------------------------------------------------------- weight gradient
// dw[t][o][i] = sum over pixels p of dout[p][o] * in[p + offset(t)][i]: per tap t a CO x CI GEMM
// over pixels. CTA (chunk, t) walks a contiguous range of rows, staging the output-gradient row
// and the shifted input row transposed ([channel][pixel]) so both fragments are 32-bit loads, and
// writes its partial sums; pgbp_conv3x3_wgrad adds the partials in chunk order (deterministic).
template <int CI, int CO>
__global__ void __launch_bounds__(256) wgrad_kernel(int64_t n, int h, int w,
                                                    const __nv_bfloat16* __restrict__ in,
                                                    const __nv_bfloat16* __restrict__ dout,
                                                    float* __restrict__ partial,
                                                    float* __restrict__ bpartial,
                                                    int64_t rows_per_cta) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ld = w + 8;
  __nv_bfloat16* sd = reinterpret_cast<__nv_bfloat16*>(smem_raw);  // [CO][ld]
  __nv_bfloat16* sx = sd + CO * ld;                                 // [CI][ld]
  constexpr int MB = CO / 16, NT = CI / 8, TPW = MB * NT / 8;
  const int t = blockIdx.y, dy = t / 3, dx = t % 3 - 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gid = lane >> 2, tig = lane & 3;
  float acc[TPW][4];
#pragma unroll
  for (int k = 0; k < TPW; ++k)
#pragma unroll
    for (int e = 0; e < 4; ++e) acc[k][e] = 0.0f;
  float bacc = 0.0f;
  const int64_t total = n * h;
  const int64_t r0 = (int64_t)blockIdx.x * rows_per_cta;
  const int64_t r1 = r0 + rows_per_cta < total ? r0 + rows_per_cta : total;
  for (int64_t r = r0; r < r1; ++r) {
    const int64_t b = r / h;
    const int y = (int)(r % h);
    const int yy = (y + dy - 1 + h) % h;
    __syncthreads();
    for (int x = threadIdx.x; x < w * CO; x += blockDim.x) {
      const int px = x / CO, o = x % CO;
      sd[o * ld + px] = dout[((b * h + y) * w + px) * CO + o];
    }
    for (int x = threadIdx.x; x < w * CI; x += blockDim.x) {
      const int px = x / CI, i = x % CI;
      const int sxp = (px + dx + w) % w;
      sx[i * ld + px] = in[((b * h + yy) * w + sxp) * CI + i];
    }
    __syncthreads();
    for (int k0 = 0; k0 < w; k0 += 16) {
#pragma unroll
      for (int k = 0; k < TPW; ++k) {
        const int tile = warp * TPW + k, mb = tile / NT, nb = tile % NT;
        const __nv_bfloat16* ra = sd + (mb * 16 + gid) * ld + k0 + 2 * tig;
        const __nv_bfloat16* rb = ra + 8 * ld;
        const uint32_t a[4] = {ld32(ra), ld32(rb), ld32(ra + 8), ld32(rb + 8)};
        const __nv_bfloat16* xb = sx + (nb * 8 + gid) * ld + k0 + 2 * tig;
        const uint32_t bb[2] = {ld32(xb), ld32(xb + 8)};
        mma_bf16(acc[k], a, bb);
      }
    }
    if (t == 4 && threadIdx.x < CO)
      for (int px = 0; px < w; ++px) bacc += __bfloat162float(sd[threadIdx.x * ld + px]);
  }
  float* dst = partial + ((int64_t)blockIdx.x * 9 + t) * CO * CI;
#pragma unroll
  for (int k = 0; k < TPW; ++k) {
    const int tile = warp * TPW + k, mb = tile / NT, nb = tile % NT;
    const int o = mb * 16 + gid, i = nb * 8 + 2 * tig;
    dst[o * CI + i] = acc[k][0];
    dst[o * CI + i + 1] = acc[k][1];
    dst[(o + 8) * CI + i] = acc[k][2];
    dst[(o + 8) * CI + i + 1] = acc[k][3];
  }
  if (t == 4 && threadIdx.x < CO) bpartial[(int64_t)blockIdx.x * CO + threadIdx.x] = bacc;
}

// out[j] = sum over c < chunks (in order) of partial[c * n + j]
__global__ void sum_chunks_kernel(const float* __restrict__ partial, int64_t chunks, int64_t n,
                                  float* __restrict__ out) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int64_t c = 0; c < chunks; ++c) s += partial[c * n + j];
    out[j] = s;
  }
}

// wt[t][i][o] = w[8 - t][o][i]
__global__ void flip_kernel(int ci, int co, const __nv_bfloat16* __restrict__ w,
                            __nv_bfloat16* __restrict__ wt) {
  for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < 9 * ci * co; x += gridDim.x * blockDim.x) {
    const int t = x / (ci * co), i = (x / co) % ci, o = x % co;
    wt[x] = w[((8 - t) * co + o) * ci + i];
  }
}

// Mean-centred squared error over groups of g values: d = (p - mean p) - (t - mean t);
// loss += sum d^2 (double, for reporting); grad = scale * 2 d (BF16).
__global__ void center_mse_kernel(int64_t groups, int g, const float* __restrict__ pred,
                                  const float* __restrict__ target,
                                  __nv_bfloat16* __restrict__ grad, double* __restrict__ loss,
                                  float scale) {
  double local = 0.0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < groups;
       k += (int64_t)gridDim.x * blockDim.x) {
    const float* p = pred + k * g;
    const float* t = target + k * g;
    float mp = 0.0f, mt = 0.0f;
    for (int s = 0; s < g; ++s) {
      mp += p[s];
      mt += t[s];
    }
    mp /= (float)g;
    mt /= (float)g;
    for (int s = 0; s < g; ++s) {
      const float d = (p[s] - mp) - (t[s] - mt);
      local += (double)d * d;
      grad[k * g + s] = __float2bfloat16(scale * 2.0f * d);
    }
  }
  for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, local);
}

// Adam on FP32 master weights; also writes their BF16 copy.
__global__ void adam_kernel(int64_t n, float* __restrict__ w, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v,
                            __nv_bfloat16* __restrict__ wb, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x) {
    const float gj = g[j];
    const float mj = b1 * m[j] + (1.0f - b1) * gj;
    const float vj = b2 * v[j] + (1.0f - b2) * gj * gj;
    m[j] = mj;
    v[j] = vj;
    const float wj = w[j] - lr * (mj / c1) / (sqrtf(vj / c2) + eps);
    w[j] = wj;
    if (wb) wb[j] = __float2bfloat16(wj);
  }
}

// ------------------------------------------------------------------------------- Potts features
// Network inputs and closed-form one-step messages of toroidal L x L Potts grids with K-state
// variables and per-edge tables J_e I_K (pgmax_gb300/warmstart/potts.py): J [n][2 L^2] (down
// factors (i, j)-(i+1, j) first, then right factors (i, j)-(i, j+1)), u [n][L^2][K]. Per variable,
// its four factors in the order down, right, up, left, with coupling J_k and the other variable's
// unaries a_k: one-step message m_k(s) = log(exp(lse(a_k)) + expm1(J_k) exp(a_k(s))), minus its
// maximum over s. x[n][i][j][64] (BF16) = (u - mean u, the four couplings, the four messages,
// zeros); m1[n][i][j][4 K] (FP32) = the four messages. One thread per (instance, variable).
template <int K>
__global__ void potts_features_kernel(int64_t n, int L, const float* __restrict__ J,
                                      const float* __restrict__ u,
                                      __nv_bfloat16* __restrict__ x, float* __restrict__ m1) {
  constexpr int kCh = 64;
  const int64_t total = n * (int64_t)L * L;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = q / ((int64_t)L * L);
    const int p = (int)(q % ((int64_t)L * L));
    const int i = p / L, j = p % L;
    const int up = ((i - 1 + L) % L) * L + j, down = ((i + 1) % L) * L + j;
    const int left = i * L + (j - 1 + L) % L, right = i * L + (j + 1) % L;
    const float* Jb = J + b * 2LL * L * L;
    const float* ub = u + b * (int64_t)L * L * K;
    const float cpl[4] = {Jb[p], Jb[L * L + p], Jb[up], Jb[L * L + left]};
    const int nb[4] = {down, right, up, left};
    float out[kCh];
    float mean = 0.0f;
#pragma unroll
    for (int s = 0; s < K; ++s) mean += ub[(int64_t)p * K + s];
    mean = mean / (float)K;
#pragma unroll
    for (int s = 0; s < K; ++s) out[s] = ub[(int64_t)p * K + s] - mean;
#pragma unroll
    for (int k = 0; k < 4; ++k) out[K + k] = cpl[k];
    float* mo = m1 + q * 4 * K;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      float a[K];
      float mx = -INFINITY;
#pragma unroll
      for (int s = 0; s < K; ++s) {
        a[s] = ub[(int64_t)nb[k] * K + s];
        mx = fmaxf(mx, a[s]);
      }
      float se = 0.0f;
#pragma unroll
      for (int s = 0; s < K; ++s) se += expf(a[s] - mx);
      const float tot = expf(mx + logf(se));  // exp(logsumexp(a)), as the torch form computes it
      const float em = expm1f(cpl[k]);
      float mk[K];
      float top = -INFINITY;
#pragma unroll
      for (int s = 0; s < K; ++s) {
        mk[s] = logf(tot + em * expf(a[s]));
        top = fmaxf(top, mk[s]);
      }
#pragma unroll
      for (int s = 0; s < K; ++s) {
        const float v = mk[s] - top;
        out[K + 4 + k * K + s] = v;
        mo[k * K + s] = v;
      }
    }
#pragma unroll
    for (int c = K + 4 + 4 * K; c < kCh; ++c) out[c] = 0.0f;
    __nv_bfloat162* xo = reinterpret_cast<__nv_bfloat162*>(x + q * kCh);
#pragma unroll
    for (int c = 0; c < kCh / 2; ++c) xo[c] = __floats2bfloat162_rn(out[2 * c], out[2 * c + 1]);
  }
}

int sm_count() {
  static int n = [] {
    int d = 0, c = 0;
    cudaGetDevice(&d);
    cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, d);
    return c > 0 ? c : 1;
  }();
  return n;
}

bool conv_shape_ok(int ci, int co) {
  return (ci == 16 && co == 64) || (ci == 64 && co == 64) || (ci == 64 && co == 32) ||
         (ci == 32 && co == 64);
}

template <int CI, int CO>
cudaError_t launch_conv(cudaStream_t s, int64_t n, int h, int w, const void* in, const void* wts,
                        const float* bias, void* out, int out_f32, int relu, const void* mask) {
  const size_t smem = ConvSmem<CI, CO>::bytes(w);
  static size_t attr = 0;
  if (smem > attr) {
    cudaError_t e = cudaFuncSetAttribute(conv3x3_kernel<CI, CO>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    attr = smem;
  }
  constexpr int kRows = ConvSmem<CI, CO>::kRows;
  const int64_t steps = n * ((h + kRows - 1) / kRows);
  int per_sm = 1;
  const int threads = 32 * kRows * (w / 16);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, conv3x3_kernel<CI, CO>, threads,
                                                    smem) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  const int64_t ctas = std::min<int64_t>(steps, (int64_t)sm_count() * per_sm);
  const int64_t per = (steps + ctas - 1) / ctas;
  conv3x3_kernel<CI, CO><<<(unsigned)((steps + per - 1) / per), threads, smem, s>>>(
      n, h, w, static_cast<const __nv_bfloat16*>(in), static_cast<const __nv_bfloat16*>(wts), bias,
      out, out_f32, relu, static_cast<const __nv_bfloat16*>(mask), per);
  return cudaGetLastError();
}

constexpr int64_t kWgradChunks = 64;

template <int CI, int CO>
cudaError_t launch_wgrad(cudaStream_t s, int64_t n, int h, int w, const void* in,
                         const void* dout, float* dw, float* db, float* ws) {
  const int64_t rows = n * h;
  const int64_t chunks = std::min<int64_t>(rows, kWgradChunks);
  const int64_t per = (rows + chunks - 1) / chunks;
  const int64_t used = (rows + per - 1) / per;
  float* partial = ws;
  float* bpartial = ws + kWgradChunks * 9 * CO * CI;
  const size_t smem = sizeof(__nv_bfloat16) * (size_t)(CO + CI) * (w + 8);
  wgrad_kernel<CI, CO><<<dim3((unsigned)used, 9), 256, smem, s>>>(
      n, h, w, static_cast<const __nv_bfloat16*>(in), static_cast<const __nv_bfloat16*>(dout),
      partial, bpartial, per);
  sum_chunks_kernel<<<(9 * CO * CI + 255) / 256, 256, 0, s>>>(partial, used, 9 * CO * CI, dw);
  if (db) sum_chunks_kernel<<<1, 256, 0, s>>>(bpartial, used, CO, db);
  return cudaGetLastError();
}

int fail(int code, const char* msg) { return pgbp::set_last_error(code, msg); }

}  // namespace

extern "C" {

int pgbp_conv3x3(void* stream, int64_t n, int h, int w, int ci, int co, const void* in,
                 const void* weights, const float* bias, void* out, int out_f32, int relu,
                 const void* mask) {
  if (!conv_shape_ok(ci, co)) return fail(PGBP_ERR_UNSUPPORTED, "conv3x3: unsupported channels");
  if (n <= 0 || h <= 0 || w <= 0 || w % 16 != 0 || w > 128)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "conv3x3: width must be a multiple of 16, at most 128");
  if (!in || !weights || !out) return fail(PGBP_ERR_INVALID_ARGUMENT, "conv3x3: null pointer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (ci == 16) e = launch_conv<16, 64>(s, n, h, w, in, weights, bias, out, out_f32, relu, mask);
  else if (ci == 32) e = launch_conv<32, 64>(s, n, h, w, in, weights, bias, out, out_f32, relu, mask);
  else if (co == 64) e = launch_conv<64, 64>(s, n, h, w, in, weights, bias, out, out_f32, relu, mask);
  else e = launch_conv<64, 32>(s, n, h, w, in, weights, bias, out, out_f32, relu, mask);
  return e == cudaSuccess ? PGBP_OK : fail(PGBP_ERR_CUDA, cudaGetErrorString(e));
}

size_t pgbp_conv3x3_wgrad_workspace(int ci, int co) {
  return sizeof(float) * (size_t)kWgradChunks * (9 * (size_t)ci * co + (size_t)co);
}

int pgbp_conv3x3_wgrad(void* stream, int64_t n, int h, int w, int ci, int co, const void* in,
                       const void* dout, float* dw, float* db, void* workspace,
                       size_t workspace_bytes) {
  if (!conv_shape_ok(ci, co)) return fail(PGBP_ERR_UNSUPPORTED, "conv3x3_wgrad: unsupported channels");
  if (n <= 0 || h <= 0 || w <= 0 || w % 16 != 0 || w > 128)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "conv3x3_wgrad: width must be a multiple of 16, <= 128");
  if (!in || !dout || !dw) return fail(PGBP_ERR_INVALID_ARGUMENT, "conv3x3_wgrad: null pointer");
  if (!workspace || workspace_bytes < pgbp_conv3x3_wgrad_workspace(ci, co))
    return fail(PGBP_ERR_WORKSPACE, "conv3x3_wgrad: workspace too small");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  float* ws = static_cast<float*>(workspace);
  cudaError_t e;
  if (ci == 16) e = launch_wgrad<16, 64>(s, n, h, w, in, dout, dw, db, ws);
  else if (ci == 32) e = launch_wgrad<32, 64>(s, n, h, w, in, dout, dw, db, ws);
  else if (co == 64) e = launch_wgrad<64, 64>(s, n, h, w, in, dout, dw, db, ws);
  else e = launch_wgrad<64, 32>(s, n, h, w, in, dout, dw, db, ws);
  return e == cudaSuccess ? PGBP_OK : fail(PGBP_ERR_CUDA, cudaGetErrorString(e));
}

int pgbp_conv3x3_flip(void* stream, int ci, int co, const void* weights, void* flipped) {
  if (!weights || !flipped || ci <= 0 || co <= 0)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "conv3x3_flip: bad argument");
  flip_kernel<<<(9 * ci * co + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      ci, co, static_cast<const __nv_bfloat16*>(weights), static_cast<__nv_bfloat16*>(flipped));
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PGBP_OK : fail(PGBP_ERR_CUDA, cudaGetErrorString(e));
}

int pgbp_center_mse(void* stream, int64_t groups, int group, const float* pred,
                    const float* target, void* grad, double* loss, float scale) {
  if (groups < 0 || group <= 0 || !pred || !target || !grad)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "center_mse: bad argument");
  if (groups == 0) return PGBP_OK;
  const int64_t blocks = std::min<int64_t>((groups + 255) / 256, (int64_t)sm_count() * 8);
  center_mse_kernel<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      groups, group, pred, target, static_cast<__nv_bfloat16*>(grad), loss, scale);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PGBP_OK : fail(PGBP_ERR_CUDA, cudaGetErrorString(e));
}

int pgbp_adam(void* stream, int64_t n, float* w, const float* g, float* m, float* v,
              void* w_bf16, float lr, float beta1, float beta2, float eps, int64_t step) {
  if (n < 0 || !w || !g || !m || !v || step < 1)
    return fail(PGBP_ERR_INVALID_ARGUMENT, "adam: bad argument");
  if (n == 0) return PGBP_OK;
  const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
  const int64_t blocks = std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 8);
  adam_kernel<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      n, w, g, m, v, static_cast<__nv_bfloat16*>(w_bf16), lr, beta1, beta2, eps, c1, c2);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PGBP_OK : fail(PGBP_ERR_CUDA, cudaGetErrorString(e));
}

int pgbp_potts_features(void* stream, int64_t n, int L, int K, const float* J, const float* u,
                        void* x, float* m1) {
  if (n <= 0 || L < 3 || K != 8) return fail(PGBP_ERR_INVALID_ARGUMENT, "supported: n > 0, L >= 3, K = 8");
  if (!J || !u || !x || !m1) return fail(PGBP_ERR_INVALID_ARGUMENT, "null data pointer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t total = n * (int64_t)L * L;
  const int64_t blocks = std::min<int64_t>((total + 255) / 256, (int64_t)sm_count() * 16);
  potts_features_kernel<8><<<(unsigned)blocks, 256, 0, s>>>(
      n, L, J, u, static_cast<__nv_bfloat16*>(x), m1);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(PGBP_ERR_CUDA, cudaGetErrorString(e));
  return PGBP_OK;
}

}  // extern "C"
