// Shared-table exp-domain update of dense K x K pairwise EnumFactors on the tensor cores
// (K = 16, 32, 64; temperature > 0; potentials shared by the batch).
//
// For a factor over variables 1 and 2 whose table psi is shared by a group of factors, the
// reference's messages (pgmax/factor/enum.py:451-475 at temperature T > 0)
//   f1[i] = T log sum_j exp((v1[i] + v2[j] + psi_ij - M1_i) / T) + M1_i - v1[i]
// are, in exact arithmetic, T log sum_j exp((v2[j] + psi_ij) / T) = T log (E u)_i + m2 + r_i with
//   r_i = max_j psi_ij,  E_ij = exp((psi_ij - r_i) / T)      per table, once per run
//   m2 = max_j v2[j],    u_j = exp((v2[j] - m2) / T)         per factor and instance
// and f2 likewise with E'_ji = exp((psi_ij - c_j) / T), c_j = max_i psi_ij, w_i from v1. A factor
// then costs 2K exponentials instead of 2K^2, and the K^2 work becomes two GEMMs per tile of 64
// (factor, instance) columns, F1 = E U and F2 = E' W (K x K by K x 64), on the tensor cores:
// mma.sync m16n8k8 TF32 with each operand split into a tf32 high part and the tf32 rounding of the
// remainder, three products per pair (lo*hi + hi*lo + hi*hi, fp32 accumulation), about 2^-21
// relative; u, w and the logarithm use the fast __expf / __logf (a few ulp): float32 accuracy,
// not bit-equal to the direct path. A sum below 1e-30 (a table row
// spanning more than about 69 T) is recomputed directly from the messages. The epilogue (damping,
// normalisation, clipping at MSG_NEG_INF, residual; pgmax/infer/bp.py:127-136) is the one of the
// dense pairwise kernel.
//
// Work split: factors of a bucket are sorted by table (plan time); a column is (factor, instance)
// with the instance innermost, and a tile is 64 consecutive columns of one group. CTAs are
// persistent over a contiguous range of tiles, reloading the table only when the group changes,
// by one bulk copy (cp.async.bulk on an mbarrier) of the run-time tables, which are built in the
// kernel's shared-memory layout.
// Four threads own a column (K / 4 states of each edge each), so a thread issues all its message
// and variable-sum loads before it uses any, and keeps the old messages in registers until the
// epilogue. The residual is folded per CTA in shared memory and written once per instance.
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <type_traits>

#include "pgbp_internal.h"

namespace pgbp {
namespace {

constexpr float kMsgNegInf = -1e32f;  // MSG_NEG_INF, pgmax/utils/__init__.py
constexpr int kCols = 64;             // (factor, instance) columns per tile
constexpr int kThreads = 256;
constexpr int kLdc = kCols + 8;       // row stride of the K x 64 operand / result tiles

__device__ __forceinline__ float maxn(float a, float b) {
  float r;
  asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}

// 2^x, PTX ex2.approx (flushes subnormal results to zero; -inf gives 0).
__device__ __forceinline__ float ex2_approx(float x) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ float minn(float a, float b) {
  float r;
  asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}

// x / t; a power-of-two t multiplies by its exact reciprocal (the same correctly rounded value).
__device__ __forceinline__ float div_t(float x, float t) {
  const unsigned u = __float_as_uint(t);
  const unsigned e = (u >> 23) & 0xffu;
  if ((u & 0x807fffffu) == 0u && e >= 2u && e <= 252u) return x * __uint_as_float((254u - e) << 23);
  return x / t;
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
  hi = to_tf32(x);
  lo = to_tf32(x - __uint_as_float(hi));
}

// ---- bulk copies into shared memory (cp.async.bulk, completion on an mbarrier)
// A wait that has not seen its copy land after the launch's limit (kWaitLimitNs unless the debug
// setting changes it) gives up: the CTA counts it in g_wait_timeouts, sets the plan's fault word
// (mapped host memory, read by pgbp_plan_check and the entry points) and stops, so a lost copy is
// an error status, not a hang and not silently wrong tables.
constexpr unsigned long long kWaitLimitNs = 2000000000ull;
__device__ unsigned long long g_wait_timeouts = 0;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One copy of `bytes` (a multiple of 16; both addresses 16-byte aligned) from global to shared
// memory, completing the current phase of `bar`. Shared-memory reads issued before it (by any
// thread, ordered by a barrier) complete before the copy writes. With `skip_copy` (a debug
// setting) the barrier is armed for the bytes but no copy is issued: its phase never completes
// and the wait for it runs out with nothing in flight.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes,
                                          uint64_t* bar, bool skip_copy) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
  if (skip_copy) return;
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

// Waits for the phase of `bar` with parity `parity` to complete; false when `limit_ns` passed
// first (measured on %globaltimer).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
                                          unsigned long long limit_ns) {
  const uint32_t addr = smem_addr(bar);
  uint64_t t0 = 0;
  for (uint32_t i = 0;; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
    if ((i & 63) == 0) {
      uint64_t now;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
      if (t0 == 0) {
        t0 = now;
      } else if (now - t0 > limit_ns) {
        return false;
      }
    }
  }
}

// D = A B + D, A 16x8 (row), B 8x8 (col), tf32 in, fp32 accumulate.
__device__ __forceinline__ void mma_tf32(float (&c)[4], const uint32_t (&a)[4],
                                         const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}


// Position of table column j in the permuted order of its 8-block.
__device__ __forceinline__ int perm8(int j) { return (j & ~7) + ((j & 3) << 1) + ((j >> 2) & 1); }

// Run-time tables of one group in the pairwise kernel's shared-memory layout (one bulk copy moves
// them there): E [K][K + 8] (row i, column perm8(j)), E' [K][K + 8] (row j, column perm8(i)), zero
// padding, row maxima r [K], column maxima c [K]. One CTA per group.
template <int K>
__global__ void __launch_bounds__(kThreads) expgemm_tables_kernel(
    const int32_t* __restrict__ grp_table, const float* __restrict__ lpc, float t,
    float* __restrict__ tables) {
  constexpr int kLde = K + 8;
  const int g = blockIdx.x;
  const float* psi = lpc + grp_table[g];
  float* out = tables + (int64_t)g * expgemm_table_floats(K);
  float *e = out, *f = out + K * kLde, *rmax = out + 2 * K * kLde, *cmax = rmax + K;
  __shared__ float rs[K], cs[K];
  for (int i = threadIdx.x; i < K; i += blockDim.x) {
    float m = -INFINITY, n = -INFINITY;
    for (int j = 0; j < K; ++j) {
      m = maxn(m, psi[i * K + j]);
      n = maxn(n, psi[j * K + i]);
    }
    rs[i] = m;
    cs[i] = n;
    rmax[i] = m;
    cmax[i] = n;
  }
  __syncthreads();
  for (int x = threadIdx.x; x < K * K; x += blockDim.x) {
    const int i = x / K, j = x % K;
    e[i * kLde + perm8(j)] = expf(div_t(psi[x] - rs[i], t));
    f[j * kLde + perm8(i)] = expf(div_t(psi[x] - cs[j], t));
  }
  for (int x = threadIdx.x; x < 2 * K * 8; x += blockDim.x) {  // padding columns
    const int r = x / 8, j = K + x % 8;
    (r < K ? e : f)[(r % K) * kLde + j] = 0.0f;
  }
}

constexpr int kMaxB = 512;  // instances whose residual a CTA folds in shared memory

struct ExpArgs {
  const int4* __restrict__ rec;           // (first edge state, first slot, var state 1, 2)
  const int32_t* __restrict__ grp_first;
  const int32_t* __restrict__ grp_count;
  const int32_t* __restrict__ grp_table;
  int n_groups;
  int64_t n_tiles, tiles_per_cta;
  int64_t B;
  const float* __restrict__ cur;
  float* __restrict__ nxt;
  const float* __restrict__ vsum;
  const float* __restrict__ lpc;          // clipped shared potentials
  const float* __restrict__ tables;
  float d, omd, t;
  unsigned* __restrict__ dacc;            // residual of this iteration, [B] float bits
  unsigned* fault;                        // the plan's fault word (mapped host memory)
  unsigned long long wait_ns;             // limit of the table wait
  int skip_copy;                          // debug: arm the table barrier, issue no copy
};

// Shared-memory layout of one CTA.
//   E, E' [K][kLde] fp32 with the columns of every 8-block in the order 0 4 1 5 2 6 3 7, so the
//     (k, k + 4) pair of an A fragment row is one 64-bit load; kLde = K + 8 puts the rows of a
//     half-warp's loads in distinct 32-byte bank groups.
//   row maxima r [K], column maxima c [K].
//   U, W as tf32 high / low parts, [K / 8][4][kLdx] uint4 = (hi(k), hi(k + 4), lo(k), lo(k + 4))
//     for k = 8 kb + tig, column n: one 128-bit load per B fragment; kLdx = 66 puts the 4 rows of
//     a quarter-warp's loads in distinct bank groups. F1 / F2 ([K][kLdc] fp32) overwrite U / W.
template <int K>
struct Smem {
  static constexpr int kLde = K + 8;
  static constexpr int kLdx = kCols + 2;
  static constexpr int kXWords = (K / 8) * 4 * kLdx * 4;  // 32-bit words of one of U, W
  static_assert(K * kLdc <= kXWords, "F1 / F2 must fit in the space of U / W");
  static constexpr int kFloats = 2 * K * kLde + 2 * K + 2 * kXWords;
  static constexpr size_t kBytes = sizeof(float) * kFloats + sizeof(unsigned) * kMaxB;
};


// State of slot i (0 .. K / 4 - 1) of the thread that owns quarter `part` of a column: the pair
// (8 kb + part, 8 kb + part + 4) for kb = i / 2, the pair the B fragment layout stores together.
__device__ __forceinline__ int state_of(int i, int part) { return (i >> 1) * 8 + part + 4 * (i & 1); }

// f for state s of one edge computed directly (the reference's formula) when the exp-domain sum
// underflows: the other variable's vtof plus row (first edge) or column s of the table.
template <int K>
__device__ float direct_message(const ExpArgs& a, int4 q, int64_t b, int s,
                               bool first_edge, int64_t table) {
  const int64_t B = a.B;
  float mx = -INFINITY;
  for (int j = 0; j < K; ++j) {
    const float v = first_edge ? a.vsum[(q.w + j) * B + b] - a.cur[(q.y + K + j) * B + b]
                               : a.vsum[(q.z + j) * B + b] - a.cur[(q.y + j) * B + b];
    const float p = first_edge ? a.lpc[table + s * K + j] : a.lpc[table + j * K + s];
    mx = maxn(mx, v + p);
  }
  float se = 0.0f;
  for (int j = 0; j < K; ++j) {
    const float v = first_edge ? a.vsum[(q.w + j) * B + b] - a.cur[(q.y + K + j) * B + b]
                               : a.vsum[(q.z + j) * B + b] - a.cur[(q.y + j) * B + b];
    const float p = first_edge ? a.lpc[table + s * K + j] : a.lpc[table + j * K + s];
    se += expf(div_t((v + p) - mx, a.t));
  }
  return a.t * logf(se) + mx;
}

// acc = T X: T (K x K fp32, permuted columns, split per fragment) times X (K x 64, split, in the
// uint4 layout). The A_lo x B_hi product accumulates apart from the other two (two chains of
// mma.sync per output tile instead of one twice as long) and is added at the end.
template <int K>
__device__ __forceinline__ void tile_gemm(const float* T, const uint4* X, int warp, int lane,
                                          float (&acc)[K / 16][4]) {
  constexpr int MB = K / 16;  // 16-row blocks; 8 warps x MB tiles = MB x 8 tiles of 16 x 8
  constexpr int kLde = Smem<K>::kLde;
  constexpr int kLdx = Smem<K>::kLdx;
  const int gid = lane >> 2, tig = lane & 3;
  const int r0 = ((warp * MB) / 8) * 16 + gid;
  float x1[MB][4];
#pragma unroll
  for (int i = 0; i < MB; ++i)
#pragma unroll
    for (int e = 0; e < 4; ++e) acc[i][e] = x1[i][e] = 0.0f;
#pragma unroll
  for (int k0 = 0; k0 < K; k0 += 8) {
    const float2 t0 = *reinterpret_cast<const float2*>(T + r0 * kLde + k0 + 2 * tig);
    const float2 t1 = *reinterpret_cast<const float2*>(T + (r0 + 8) * kLde + k0 + 2 * tig);
    uint32_t ah[4], al[4];
    split_tf32(t0.x, ah[0], al[0]);  // (r0, k0 + tig)
    split_tf32(t1.x, ah[1], al[1]);  // (r0 + 8, k0 + tig)
    split_tf32(t0.y, ah[2], al[2]);  // (r0, k0 + tig + 4)
    split_tf32(t1.y, ah[3], al[3]);  // (r0 + 8, k0 + tig + 4)
#pragma unroll
    for (int i = 0; i < MB; ++i) {
      const int nb = (warp * MB + i) % 8;
      const uint4 v = X[((k0 / 8) * 4 + tig) * kLdx + nb * 8 + gid];
      const uint32_t bh[2] = {v.x, v.y};
      const uint32_t bl[2] = {v.z, v.w};
      mma_tf32(x1[i], al, bh);
      mma_tf32(acc[i], ah, bl);
      mma_tf32(acc[i], ah, bh);
    }
  }
#pragma unroll
  for (int i = 0; i < MB; ++i)
#pragma unroll
    for (int e = 0; e < 4; ++e) acc[i][e] += x1[i][e];
}

template <int K>
__device__ __forceinline__ void store_acc(float* X, int warp, int lane,
                                          const float (&acc)[K / 16][4]) {
  constexpr int MB = K / 16;
  const int gid = lane >> 2, tig = lane & 3;
  const int r0 = ((warp * MB) / 8) * 16 + gid;
#pragma unroll
  for (int i = 0; i < MB; ++i) {
    const int c0 = ((warp * MB + i) % 8) * 8 + 2 * tig;
    X[r0 * kLdc + c0] = acc[i][0];
    X[r0 * kLdc + c0 + 1] = acc[i][1];
    X[(r0 + 8) * kLdc + c0] = acc[i][2];
    X[(r0 + 8) * kLdc + c0 + 1] = acc[i][3];
  }
}

__device__ __forceinline__ float max4(float x) {  // maximum over the 4 threads of a column
  x = maxn(x, __shfl_xor_sync(0xffffffffu, x, 1));
  return maxn(x, __shfl_xor_sync(0xffffffffu, x, 2));
}

// B1: one instance (slot s of the batch at s), which saves the 64-bit index arithmetic.
template <int K, bool B1>
__global__ void __launch_bounds__(kThreads, 2) expgemm_pairwise_kernel(ExpArgs a) {
  extern __shared__ __align__(16) float sm[];
  constexpr int kLde = Smem<K>::kLde;
  constexpr int kLdx = Smem<K>::kLdx;
  constexpr int SPT = K / 4;  // states of each edge per thread (state_of)
  float* s_e = sm;                    // E  [K][kLde], permuted columns
  float* s_f = s_e + K * kLde;        // E' [K][kLde]
  float* s_r = s_f + K * kLde;        // row maxima, then column maxima
  float* s_c = s_r + K;
  uint4* s_u = reinterpret_cast<uint4*>(s_c + K);           // U (split), then F1
  uint4* s_w = s_u + Smem<K>::kXWords / 4;                  // W (split), then F2
  float* s_f1 = reinterpret_cast<float*>(s_u);
  float* s_f2 = reinterpret_cast<float*>(s_w);
  unsigned* s_res = reinterpret_cast<unsigned*>(s_w + Smem<K>::kXWords / 4);
  __shared__ int s_group;
  __shared__ int64_t s_tile0;
  __shared__ __align__(8) uint64_t s_bar;  // completion of the table copy

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = threadIdx.x >> 2, part = threadIdx.x & 3;  // column of the tile, quarter of it
  const int64_t B = B1 ? 1 : a.B;
  const bool fold = B <= kMaxB;
  if (fold)
    for (int64_t x = threadIdx.x; x < B; x += kThreads) s_res[x] = 0u;
  const int64_t t_begin = (int64_t)blockIdx.x * a.tiles_per_cta;
  const int64_t t_end = t_begin + a.tiles_per_cta < a.n_tiles ? t_begin + a.tiles_per_cta : a.n_tiles;
  int loaded = -1;
  uint32_t phase = 0;    // parity of s_bar's current phase
  bool pending = false;  // a table copy this thread has not yet waited for
  if (threadIdx.x == 0) {
    s_group = 0;
    s_tile0 = 0;
    mbar_init(&s_bar);
  }
  __syncthreads();
  for (int64_t tile = t_begin; tile < t_end; ++tile) {
    // the group of this tile (the tiles of a CTA are visited in order)
    if (threadIdx.x == 0) {
      int g = s_group;
      int64_t t0 = s_tile0;
      while (g < a.n_groups) {
        const int64_t nt = ((int64_t)a.grp_count[g] * B + kCols - 1) / kCols;
        if (tile < t0 + nt) break;
        t0 += nt;
        ++g;
      }
      s_group = g;
      s_tile0 = t0;
    }
    __syncthreads();
    const int g = s_group;
    const int64_t first = a.grp_first[g];
    const int64_t cols = (int64_t)a.grp_count[g] * B;
    const int64_t c0 = (tile - s_tile0) * kCols;
    const int ncols = (int)(cols - c0 < kCols ? cols - c0 : kCols);
    const int64_t table = a.grp_table[g];
    if (g != loaded) {
      // E, E', r, c of the group land in s_e .. s_c with one bulk copy (the table block is laid
      // out as they are), overlapping this tile's message loads; waited for before the GEMMs
      if (threadIdx.x == 0)
        bulk_load(s_e, a.tables + (int64_t)g * expgemm_table_floats(K),
                  (uint32_t)(sizeof(float) * expgemm_table_floats(K)), &s_bar, a.skip_copy != 0);
      pending = true;
      loaded = g;
    }
    // ---- load: every message and variable sum of this thread's states first, then the maxima
    const bool active = c < ncols;
    int64_t b = 0;
    int4 q = make_int4(0, 0, 0, 0);
    float o1[SPT], o2[SPT], v1[SPT], v2[SPT];
    float m1 = -INFINITY, m2 = -INFINITY;
    if (active) {
      const int64_t col = c0 + c;
      b = B1 ? 0 : col % B;
      q = a.rec[first + (B1 ? col : col / B)];
#pragma unroll
      for (int i = 0; i < SPT; ++i) {
        const int s = state_of(i, part);
        if (B1) {
          o1[i] = a.cur[q.y + s];
          o2[i] = a.cur[q.y + K + s];
          v1[i] = a.vsum[q.z + s];
          v2[i] = a.vsum[q.w + s];
        } else {
          o1[i] = a.cur[(q.y + s) * B + b];
          o2[i] = a.cur[(q.y + K + s) * B + b];
          v1[i] = a.vsum[(q.z + s) * B + b];
          v2[i] = a.vsum[(q.w + s) * B + b];
        }
      }
#pragma unroll
      for (int i = 0; i < SPT; ++i) {
        v1[i] -= o1[i];
        v2[i] -= o2[i];
        m1 = maxn(m1, v1[i]);
        m2 = maxn(m2, v2[i]);
      }
    }
    m1 = max4(m1);
    m2 = max4(m2);
    // u, w in [0, 1]: the fast exponential (about 2 ulp) keeps the sums at float32 accuracy.
    // Slots 2 kb and 2 kb + 1 are the states (8 kb + part, 8 kb + part + 4): one 128-bit store each
#pragma unroll
    for (int kb = 0; kb < K / 8; ++kb) {
      uint32_t h0, l0, h1, l1;
      split_tf32(active ? __expf(div_t(v1[2 * kb] - m1, a.t)) : 0.0f, h0, l0);
      split_tf32(active ? __expf(div_t(v1[2 * kb + 1] - m1, a.t)) : 0.0f, h1, l1);
      s_w[(kb * 4 + part) * kLdx + c] = make_uint4(h0, h1, l0, l1);
      split_tf32(active ? __expf(div_t(v2[2 * kb] - m2, a.t)) : 0.0f, h0, l0);
      split_tf32(active ? __expf(div_t(v2[2 * kb + 1] - m2, a.t)) : 0.0f, h1, l1);
      s_u[(kb * 4 + part) * kLdx + c] = make_uint4(h0, h1, l0, l1);
    }
    int lost = 0;
    if (pending) {
      lost = mbar_wait(&s_bar, phase, a.wait_ns) ? 0 : 1;
      phase ^= 1u;
      pending = false;
    }
    if (__syncthreads_or(lost)) {
      // the tables never arrived: record the fault and stop without touching them; a copy that
      // may still be in flight gets one more bounded wait before the CTA's shared memory goes
      if (threadIdx.x == 0) {
        atomicAdd(&g_wait_timeouts, 1ull);
        if (a.fault != nullptr) {
          *reinterpret_cast<volatile unsigned*>(a.fault) = 1u;
          __threadfence_system();
        }
        if (!a.skip_copy) mbar_wait(&s_bar, phase ^ 1u, a.wait_ns);
      }
      return;
    }
    // ---- F1 = E U, F2 = E' W on the tensor cores, one accumulator set live at a time (each
    // result overwrites its own operand once every warp is done reading it)
    {
      float acc[K / 16][4];
      tile_gemm<K>(s_e, s_u, warp, lane, acc);
      __syncthreads();
      store_acc<K>(s_f1, warp, lane, acc);
      tile_gemm<K>(s_f, s_w, warp, lane, acc);
      __syncthreads();
      store_acc<K>(s_f2, warp, lane, acc);
    }
    __syncthreads();
    // ---- epilogue: messages, damping, normalisation, clipping, residual
    float x1 = -INFINITY, x2 = -INFINITY;
    if (active) {
#pragma unroll
      for (int i = 0; i < SPT; ++i) {
        const int s = state_of(i, part);
        const float e1 = s_f1[s * kLdc + c], e2 = s_f2[s * kLdc + c];
        // the sums are >= 1e-30 here: the fast logarithm's absolute error is about 4e-7
        const float f1 = e1 >= 1e-30f ? (a.t * __logf(e1) + m2) + s_r[s]
                                      : direct_message<K>(a, q, b, s, true, table);
        const float f2 = e2 >= 1e-30f ? (a.t * __logf(e2) + m1) + s_c[s]
                                      : direct_message<K>(a, q, b, s, false, table);
        v1[i] = a.d * o1[i] + a.omd * f1;  // v1 / v2 now hold the damped messages
        v2[i] = a.d * o2[i] + a.omd * f2;
        x1 = maxn(x1, v1[i]);
        x2 = maxn(x2, v2[i]);
      }
    }
    x1 = max4(x1);
    x2 = max4(x2);
    float dmax = 0.0f;
    if (active) {
#pragma unroll
      for (int i = 0; i < SPT; ++i) {
        const int s = state_of(i, part);
        const float y1 = maxn(v1[i] - x1, kMsgNegInf);
        const float y2 = maxn(v2[i] - x2, kMsgNegInf);
        if (B1) {
          a.nxt[q.y + s] = y1;
          a.nxt[q.y + K + s] = y2;
        } else {
          a.nxt[(q.y + s) * B + b] = y1;
          a.nxt[(q.y + K + s) * B + b] = y2;
        }
        dmax = maxn(dmax, fabsf(y1 - o1[i]));
        dmax = maxn(dmax, fabsf(y2 - o2[i]));
      }
    }
    dmax = max4(dmax);
    if (active && part == 0 && a.dacc != nullptr) {
      if (fold) atomicMax(s_res + b, __float_as_uint(dmax));
      else atomicMax(a.dacc + b, __float_as_uint(dmax));
    }
    __syncthreads();
  }
  if (fold && a.dacc != nullptr) {
    for (int64_t x = threadIdx.x; x < B; x += kThreads)
      if (s_res[x] != 0u) atomicMax(a.dacc + x, s_res[x]);
  }
}

template <int K, bool B1>
cudaError_t set_smem_attr() {
  static cudaError_t once = cudaFuncSetAttribute(
      expgemm_pairwise_kernel<K, B1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
      (int)Smem<K>::kBytes);
  return once;
}

template <int K, bool B1>
cudaError_t launch_b(const Plan& p, const PairwiseBucket& q, cudaStream_t s, const ExpArgs& base) {
  cudaError_t e = set_smem_attr<K, B1>();
  if (e != cudaSuccess) return e;
  static int per_sm = -1;
  if (per_sm < 0) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, expgemm_pairwise_kernel<K, B1>, kThreads,
                                                      Smem<K>::kBytes) != cudaSuccess)
      n = 1;
    per_sm = std::max(n, 1);
  }
  ExpArgs a = base;
  int64_t tiles = 0;
  for (int64_t c : q.grp_count_host) tiles += (c * a.B + kCols - 1) / kCols;
  if (tiles == 0) return cudaSuccess;
  const int64_t ctas = std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)p.sm_count * per_sm));
  a.n_tiles = tiles;
  a.tiles_per_cta = (tiles + ctas - 1) / ctas;
  const int64_t grid = (tiles + a.tiles_per_cta - 1) / a.tiles_per_cta;
  expgemm_pairwise_kernel<K, B1><<<(unsigned)grid, kThreads, Smem<K>::kBytes, s>>>(a);
  return cudaGetLastError();
}

template <int K>
cudaError_t launch(const Plan& p, const PairwiseBucket& q, cudaStream_t s, const ExpArgs& a) {
  return a.B == 1 ? launch_b<K, true>(p, q, s, a) : launch_b<K, false>(p, q, s, a);
}

// ============================================================================ tcgen05 path
// K = 64, one instance (B = 1; batches keep the kernel above). The same arithmetic as above with
// the products on the fifth-generation tensor cores: tcgen05.mma kind::tf32, A and B operands in
// shared memory (128-byte swizzled, K-major), accumulators in tensor memory (TMEM), and the work
// of a tile split over specialised warps so that loads, the products and the epilogue of
// consecutive units overlap.
//   The CTAs come in pairs over the same range of tiles (a tile = up to 128 consecutive factors
//   of one group); CTA 2 r computes the messages to variable 1 of range r, CTA 2 r + 1 those to
//   variable 2, so a CTA holds one direction's tables and the two CTAs of a pair read each
//   message row at about the same time (one DRAM read, one L2 hit). Unit u of a CTA = its tile u:
//     direction 0: D[c][i] = sum_j U[c][j] E[i][j], U from variable 2 (the messages to 1);
//     direction 1: D[c][j] = sum_i W[c][i] E'[j][i], W from variable 1 (the messages to 2).
//   M = 128 columns, N = 64 states, K = 64 states in 8 steps of 8; three products per step
//   (hi x hi, hi x lo, lo x hi of the tf32 splits), float32 accumulation in TMEM.
//   * producer warps 4-14, two steps per unit, so that the copies of unit u are in flight while
//     unit u - 1 is converted and unit u - 2 multiplied:
//       copy u: cp.async of each column's other-edge message and of the other variable's sums
//       into raw buffer u & 1 (16-byte chunks at the operand's swizzled positions);
//       convert u - 1: a thread per (column cc, half of the states) in warps 4-11 (the TMEM lane
//       quadrant of its warp): vtof = sums - message, the column maximum (the two halves swap
//       theirs through their raw rows), u = exp((vtof - max) / T) split into tf32 high and low
//       parts stored into TMEM operand buffer (u - 1) & 1 with tcgen05.st; the column maxima and
//       the group's table maxima are left for the epilogue;
//   * MMA warp 15: loads the group's two tables of its direction (high and low tf32 parts, built
//     once per run in the swizzled layout) with one bulk copy when the group changes, then
//     issues the 24 tcgen05.mma of the unit (A from TMEM, B from shared memory) into TMEM
//     accumulator stage u & 1 and commits them;
//   * epilogue warps 0-3 (a thread per column = TMEM lane): fetch the columns' old messages of
//     the next unit by cp.async into a staging buffer while this unit is finished: tcgen05.ld of
//     the sums, log, damping, normalisation, clipping and the residual; the new messages are
//     written to the staging rows and stored by the warp with lanes across states.
// Handshakes (mbarriers): raw_full[2] (cp.async completion) / raw_free[2] (conversion done),
// a_full[2] (producers -> MMA), mma_done[2] (tcgen05.commit -> producers, epilogue, table
// reload), tmem_free[2] (epilogue -> MMA), meta_full[2] / meta_free[2] (producers <-> epilogue:
// column and table maxima), own_full[2] / own_free[2] (producers <-> epilogue: message slots). Every wait is bounded; the first that runs
// out sets a CTA abort flag that ends every other wait, the CTA records the fault and stops, and
// TMEM is freed after the last committed products have completed.
namespace tc {

constexpr int K = 64;
constexpr int kM = 128;                  // columns per tile (the MMA's M)
constexpr int kEpiWarps = 8;             // warps 0-7: TMEM lane quadrant w % 4, states 32 (w / 4) ..
constexpr int kProdWarps = 11;           // warps 8-18
constexpr int kMmaWarp = 19;
constexpr int kThreads = 32 * 20;        // five warps per SM sub-partition: 96 registers each
constexpr int kColsPerProd = (kM + kProdWarps - 1) / kProdWarps;  // 12 columns per producer warp
constexpr int kCvtWarps = kM / 16;       // producer warps that convert: 16 columns x 2 halves each
static_assert(kCvtWarps <= kProdWarps, "converting warps");
static_assert(kColsPerProd % 2 == 0, "producer columns come in half-warp pairs");
// tensor memory: accumulator stage s at columns 64 s (0-127); operand buffer b at 128 + 128 b,
// high part then low part (64 columns each); the epilogue's half-row maxima at 384 + 2 s + half
constexpr uint32_t kTmemCols = 512;
constexpr uint32_t kTmemA = 128;
constexpr uint32_t kTmemX = 384;
// instruction descriptor: D f32 (bits 4-5 = 1), A and B tf32 (bits 7-9, 10-12 = 2), both
// K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(K >> 3) << 17) |
                            ((uint32_t)(kM >> 4) << 24);

// shared memory, byte offsets from a 1024-byte aligned base
constexpr int kMatBytes = K * K * 4;                 // one 64 x 64 tf32 table: 16 KB
constexpr int kTabBytes = 2 * kMatBytes;             // this direction's table: high, low parts
constexpr int kABytes = kM * K * 4;                  // one 128 x 64 float matrix: 32 KB
constexpr int kABufBytes = 2 * kABytes;              // a raw buffer: other messages, sums
constexpr int kOffA = kTabBytes;                     // 2 raw buffers (swizzled like an operand)
constexpr int kOffStg = kOffA + 2 * kABufBytes;      // 2 x [kM][K] floats, rows XOR-swizzled
constexpr int kStgBytes = kM * K * 4;
constexpr int kOffM = kOffStg + 2 * kStgBytes;       // 2 x [kM] maxima of the other vtof
constexpr int kOffR = kOffM + 2 * kM * 4;            // 2 x [K] table row / column maxima
constexpr int kOffOwn = kOffR + 2 * K * 4;           // 2 x [kM] slot of each column's message
constexpr int kOffBar = kOffOwn + 2 * kM * 4;
enum { kBarTab = 0, kBarAFull0, kBarAFull1, kBarMma0, kBarMma1, kBarTmem0, kBarTmem1,
       kBarMetaFull0, kBarMetaFull1, kBarMetaFree0, kBarMetaFree1, kBarOwnFull0, kBarOwnFull1,
       kBarOwnFree0, kBarOwnFree1, kBarRawFull0, kBarRawFull1, kBarRawFree0, kBarRawFree1,
       kNumBars };
constexpr int kOffMisc = kOffBar + kNumBars * 8;     // TMEM address, abort flags, residual
constexpr int kSmemBytes = kOffMisc + 16;
// the dynamic shared memory starts at the CTA's shared window (no static shared memory), which
// the kernel checks to be 1024-byte aligned (the swizzled operands need it)
static_assert(kSmemBytes <= 227 * 1024, "shared memory");
static_assert(kOffBar % 8 == 0 && kOffStg % 16 == 0 && kOffA % 1024 == 0, "alignment");

// Staging rows: the 16-byte chunk q (states 4 q .. 4 q + 3) of row c at float c * K + 4 (q ^ (c &
// 7)), so that eight threads reading chunk q of eight consecutive rows, and a half-warp reading
// the 16 chunks of one row, each take the fewest shared-memory wavefronts.
__device__ __forceinline__ int stg_chunk(int c, int q) { return c * K + ((q ^ (c & 7)) << 2); }

// floats of one group's tables in the run workspace: the four matrices, then r [K], c [K]
constexpr int64_t kTabFloats = 4LL * K * K + 2LL * K;

// Byte offset of element (r, k) of an R x 64 tf32 matrix in the 128-byte swizzled K-major layout:
// two 32-element-wide atoms along k, R x 128 B each; row r at r * 128 B (8-row groups 1024 B
// apart); the 16-byte chunk k / 4 of a row XOR row % 8.
__host__ __device__ __forceinline__ uint32_t sw128(int r, int k, int R) {
  const int atom = k >> 5, kk = k & 31;
  return (uint32_t)(atom * (R * 128) + r * 128 + ((((kk >> 2) ^ r) & 7) << 4) + ((kk & 3) << 2));
}

// Shared-memory matrix descriptor (tcgen05): start address >> 4 (bits 0-13), leading byte offset
// (bits 16-29; unused by swizzled K-major layouts), stride byte offset >> 4 (bits 32-45: 1024 B
// between 8-row groups), version 1 (bits 46-47), layout 128-byte swizzle (bits 61-63 = 2).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Descriptor of k-step ks (elements 8 ks .. 8 ks + 7) of an R-row matrix at `base`.
__device__ __forceinline__ uint64_t kstep_desc(uint32_t base, int ks, int R) {
  return sdesc(base + (uint32_t)((ks >> 2) * (R * 128) + (ks & 3) * 32));
}

// D (+)= A B^T for one k-step: A in tensor memory (128 lanes = rows, 8 columns = the k-step's
// elements), B from a shared-memory descriptor, D in tensor memory.
__device__ __forceinline__ void mma_tf32_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t b,
                                            uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}" ::"r"(d_tmem),
      "r"(a_tmem), "l"(b), "r"(kIdesc), "r"(acc)
      : "memory");
}

// 16 consecutive 32-bit columns of the warp's 32 TMEM lanes (thread = lane) from registers.
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]),
      "r"(r[15])
      : "memory");
}

// One 32-bit column of the warp's 32 TMEM lanes from a register.
__device__ __forceinline__ void tmem_st1(uint32_t taddr, uint32_t r) {
  asm volatile("tcgen05.st.sync.aligned.32x32b.x1.b32 [%0], {%1};" ::"r"(taddr), "r"(r)
               : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 16 consecutive fp32 columns of the warp's 32 TMEM lanes (thread = lane), without the wait: a
// batch of loads completes at one tcgen05.wait::ld, which must come before `r` is read.
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

__device__ __forceinline__ void bar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void bar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// Bounded wait for the phase of `bar` with parity `parity`: false when the flag `abort` is set or
// the limit passes (then this wait sets the flag). A role that is rarely on the critical path
// passes `sleep_ns` > 0 to sleep between polls, leaving the issue slots to the warps that work.
__device__ __forceinline__ bool wait(uint64_t* bar, uint32_t parity, unsigned long long limit_ns,
                                     volatile int* abort, unsigned sleep_ns = 0) {
  const uint32_t addr = smem_addr(bar);
  uint64_t t0 = 0;
  for (uint32_t i = 0;; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(addr), "r"(parity)
        : "memory");
    if (done) return true;
    if (sleep_ns != 0) __nanosleep(sleep_ns);
    if ((i & 15) == 0) {
      if (*abort) return false;
      uint64_t now;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(now));
      if (t0 == 0) {
        t0 = now;
      } else if (now - t0 > limit_ns) {
        *abort = 1;
        return false;
      }
    }
  }
}

__device__ __forceinline__ float warp_max(float x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = maxn(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}

// Named barrier `id` over `count` threads (a multiple of 32).
__device__ __forceinline__ void named_bar_sync(int id, int count) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// AND of `pred` over the `count` threads of named barrier `id`; each of them gets the result.
__device__ __forceinline__ bool named_bar_and(int id, int count, bool pred) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.and.pred q, %2, %3, p;\n"
      " selp.u32 %0, 1, 0, q;\n}"
      : "=r"(r)
      : "r"((uint32_t)pred), "r"(id), "r"(count)
      : "memory");
  return r != 0u;
}

// Run-time tables of one group for this path: E hi, E lo (rows i, k = j), E' hi, E' lo (rows j,
// k = i) in the swizzled layout above, then the row maxima r [K] and the column maxima c [K].
__global__ void __launch_bounds__(256) tables_kernel(const int32_t* __restrict__ grp_table,
                                                     const float* __restrict__ lpc, float t,
                                                     float* __restrict__ tables) {
  const int g = blockIdx.x;
  const float* psi = lpc + grp_table[g];
  float* out = tables + (int64_t)g * kTabFloats;
  char* mats = reinterpret_cast<char*>(out);
  float* rmax = out + 4 * K * K;
  float* cmax = rmax + K;
  __shared__ float rs[K], cs[K];
  for (int i = threadIdx.x; i < K; i += blockDim.x) {
    float m = -INFINITY, n = -INFINITY;
    for (int j = 0; j < K; ++j) {
      m = maxn(m, psi[i * K + j]);
      n = maxn(n, psi[j * K + i]);
    }
    rs[i] = m;
    cs[i] = n;
    rmax[i] = m;
    cmax[i] = n;
  }
  __syncthreads();
  for (int x = threadIdx.x; x < K * K; x += blockDim.x) {
    const int i = x / K, j = x % K;
    uint32_t h, l;
    split_tf32(expf(div_t(psi[x] - rs[i], t)), h, l);
    *reinterpret_cast<uint32_t*>(mats + 0 * kMatBytes + sw128(i, j, K)) = h;
    *reinterpret_cast<uint32_t*>(mats + 1 * kMatBytes + sw128(i, j, K)) = l;
    split_tf32(expf(div_t(psi[x] - cs[j], t)), h, l);
    *reinterpret_cast<uint32_t*>(mats + 2 * kMatBytes + sw128(j, i, K)) = h;
    *reinterpret_cast<uint32_t*>(mats + 3 * kMatBytes + sw128(j, i, K)) = l;
  }
}

// One fp32 column of the warp's 32 TMEM lanes (thread = lane).
__device__ __forceinline__ float tmem_ld1(uint32_t taddr) {
  uint32_t r;
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];" : "=r"(r) : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
  return __uint_as_float(r);
}

// The epilogue's damped message for a state from the sum E u (>= 1e-30): d o + (1 - d) f with
// f = T log(sum) + max of the other vtof + table maximum, as
// fma(d, o, fma((1 - d) T ln 2, log2(sum), (1 - d) max + (1 - d) table maximum)).
__device__ __forceinline__ float epi_message(const ExpArgs& a, float atl2, float sum,
                                             float omd_mo_rr, float o) {
  float lg;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(lg) : "f"(sum));   // sum is normal on this path
  return __fmaf_rn(a.d, o, __fmaf_rn(atl2, lg, omd_mo_rr));
}

// The damped message of state st of a column whose sum E u fell below 1e-30 or is not a number:
// the reference's formula (direct_message). Out of line, so that the common path stays compact.
__device__ __noinline__ float epi_message_slow(const ExpArgs& a, int4 q, int st, bool first_edge,
                                               int64_t table, float o) {
  const float f = direct_message<K>(a, q, 0, st, first_edge, table);
  return a.d * o + a.omd * f;
}

// Tile `tile` of the CTA's walk: its group (cursor g, first tile t0 of g).
// (Tile indices fit in int32: the launcher takes this kernel only below 2^31 tiles.)
struct TileCursor {
  int g = -1;
  int count = 0;        // columns of group g
  int t0 = 0, t1 = 0;   // group g's tiles are t0 .. t1 - 1
  // a group's column count is loaded once, when the walk enters the group
  __device__ void seek(const ExpArgs& a, int tile) {
    while (tile >= t1 && g + 1 < a.n_groups) {
      ++g;
      t0 = t1;
      count = a.grp_count[g];
      t1 = t0 + (count + kM - 1) / kM;
    }
  }
  __device__ int c0(int tile) const { return (tile - t0) * kM; }
  __device__ int ncols(int tile) const {
    const int left = count - (tile - t0) * kM;
    return left < kM ? left : kM;
  }
};

__global__ void __launch_bounds__(kThreads, 1) pairwise_kernel(ExpArgs a, const float* tc_tables) {
  extern __shared__ __align__(1024) unsigned char dyn[];
  unsigned char* sm = dyn;
  const uint32_t s_base = smem_addr(sm);
  if ((s_base & 1023u) != 0u) {  // not expected: reported as a fault, nothing touched
    if (threadIdx.x == 0 && a.fault != nullptr) {
      *reinterpret_cast<volatile unsigned*>(a.fault) = 1u;
      __threadfence_system();
    }
    return;
  }
  uint64_t* bars = reinterpret_cast<uint64_t*>(sm + kOffBar);
  uint32_t* s_tmem = reinterpret_cast<uint32_t*>(sm + kOffMisc);
  volatile int* s_abort = reinterpret_cast<volatile int*>(sm + kOffMisc + 4);
  unsigned* s_res = reinterpret_cast<unsigned*>(sm + kOffMisc + 8);
  volatile int* s_drain = reinterpret_cast<volatile int*>(sm + kOffMisc + 12);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned long long lim = a.wait_ns;

  // the pair of CTAs over range blockIdx.x / 2: direction blockIdx.x & 1
  const int dir = (int)(blockIdx.x & 1u);
  const int64_t t_begin = (int64_t)(blockIdx.x >> 1) * a.tiles_per_cta;
  const int64_t t_end =
      t_begin + a.tiles_per_cta < a.n_tiles ? t_begin + a.tiles_per_cta : a.n_tiles;
  const int64_t n_units = t_end > t_begin ? t_end - t_begin : 0;

  if (threadIdx.x == 0) {
    bar_init(&bars[kBarTab], 1);
    bar_init(&bars[kBarAFull0], 32 * kProdWarps);
    bar_init(&bars[kBarAFull1], 32 * kProdWarps);
    bar_init(&bars[kBarMma0], 1);
    bar_init(&bars[kBarMma1], 1);
    bar_init(&bars[kBarTmem0], 32 * kEpiWarps);
    bar_init(&bars[kBarTmem1], 32 * kEpiWarps);
    bar_init(&bars[kBarMetaFull0], 32 * kProdWarps);
    bar_init(&bars[kBarMetaFull1], 32 * kProdWarps);
    bar_init(&bars[kBarMetaFree0], 32 * kEpiWarps);
    bar_init(&bars[kBarMetaFree1], 32 * kEpiWarps);
    bar_init(&bars[kBarOwnFull0], 32 * kProdWarps);
    bar_init(&bars[kBarOwnFull1], 32 * kProdWarps);
    bar_init(&bars[kBarOwnFree0], 32 * kEpiWarps);
    bar_init(&bars[kBarOwnFree1], 32 * kEpiWarps);
    bar_init(&bars[kBarRawFull0], 32 * kProdWarps);   // cp.async completion, one per thread
    bar_init(&bars[kBarRawFull1], 32 * kProdWarps);
    bar_init(&bars[kBarRawFree0], 32 * kCvtWarps);
    bar_init(&bars[kBarRawFree1], 32 * kCvtWarps);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    *s_abort = 0;
    *s_res = 0u;
    *s_drain = 0;
  }
  if (warp == kMmaWarp) {  // the whole warp allocates (and later frees) the TMEM columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(s_tmem)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    fence_before_sync();
  }
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *s_tmem;
  const float* tab_g0 = tc_tables;  // group g's block: tc_tables + g * kTabFloats

  if (warp >= kEpiWarps && warp < kEpiWarps + kProdWarps) {
    // ------------------------------------------------------------------ producers
    // Step u copies unit u (warp p takes columns p, p + 11, ... of the tile, lanes across
    // states; nothing passes through registers) and converts unit u - 1 in place (warps 0-7 of
    // the producers, a thread per (column cc = 16 p + lane % 16, half ch = lane / 16 of the
    // states)).
    const int p = warp - kEpiWarps;
    struct Unit {       // a tile as the producers see it
      int ncols, g;     // columns, group
      int qy, qv;       // the record of column p + 11 lane (lane < 12): message pair, other sums
      float r0, r1;     // warp 8: the group's table maxima of states lane, lane + 32
    };
    TileCursor cur;
    auto tile_info = [&](int64_t tile64) {
      Unit x;
      const int tile = (int)tile64;
      cur.seek(a, tile);
      x.g = cur.g;
      const int64_t c0 = cur.c0(tile);
      x.ncols = cur.ncols(tile);
      int4 q = make_int4(0, 0, 0, 0);
      if (lane < kColsPerProd && p + kProdWarps * lane < x.ncols)
        q = a.rec[a.grp_first[x.g] + c0 + p + kProdWarps * lane];
      x.qy = q.y;
      x.qv = dir == 0 ? q.w : q.z;
      x.r0 = x.r1 = 0.0f;
      if (p == kCvtWarps) {  // this direction's table maxima: r (to variable 1) or c (to 2)
        const float* mx = tab_g0 + (int64_t)x.g * kTabFloats + 4 * K * K + dir * K;
        x.r0 = mx[lane];
        x.r1 = mx[lane + 32];
      }
      return x;
    };
    // u = exp((t - m) / T) = 2^(t c2 - m c2), c2 = log2(e) / T: one fma and ex2.approx
    const float c2 = 1.4426950408889634f / a.t;
    // converting warp p (< 8) takes TMEM lane quadrant p % 4 (the one its warp may access):
    // thread = (column cc = 32 (p % 4) + lane, half ch = p / 4 of the states)
    const int cc = 32 * (p & 3) + lane, ch = (p >> 2) & 1;
    const uint32_t cvt_off = (uint32_t)(ch * (kM * 128) + cc * 128);
    const uint32_t mx_off = (uint32_t)(cc * 128 + ((cc & 7) << 4));   // chunk 0 of the row
    // vtof = sums - message of the pair at (cc, ch) of raw buffer `buf`, the column maximum (the
    // two halves exchange theirs through their rows, dead once read), u = exp((vtof - max) / T)
    // split into tf32 parts written to TMEM operand buffer `ab`; the raw rows are released
    auto convert = [&](unsigned char* buf, int ab, int ncols, float* meta_m,
                       uint64_t* raw_free) {
      float t[32];
      float mx = -INFINITY;
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) {
        const uint32_t off = cvt_off + (uint32_t)(((jj ^ cc) & 7) << 4);
        const float4 o = *reinterpret_cast<const float4*>(buf + off);
        const float4 v = *reinterpret_cast<const float4*>(buf + kABytes + off);
        t[4 * jj + 0] = v.x - o.x;
        t[4 * jj + 1] = v.y - o.y;
        t[4 * jj + 2] = v.z - o.z;
        t[4 * jj + 3] = v.w - o.w;
#pragma unroll
        for (int q = 0; q < 4; ++q) mx = maxn(mx, t[4 * jj + q]);
      }
      *reinterpret_cast<float*>(buf + ch * (kM * 128) + mx_off) = mx;
      named_bar_sync(2, 32 * kCvtWarps);
      const float m = maxn(mx, *reinterpret_cast<const float*>(buf + (ch ^ 1) * (kM * 128) + mx_off));
      bar_arrive(raw_free);
      const bool act = cc < ncols;
      const float mc2 = -m * c2;
      const uint32_t ta =
          tmem + ((uint32_t)(32 * (p & 3)) << 16) + kTmemA + (uint32_t)(ab * 128 + 32 * ch);
#pragma unroll
      for (int k16 = 0; k16 < 2; ++k16) {
        uint32_t h[16], l[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) {
          const float z = act ? __fmaf_rn(t[16 * k16 + k], c2, mc2) : -INFINITY;
          split_tf32(ex2_approx(z), h[k], l[k]);   // a column past the tile's end: zeros
        }
        tmem_st16(ta + 16u * k16, h);
        tmem_st16(ta + 64u + 16u * k16, l);
      }
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      if (ch == 0 && act) meta_m[cc] = m;
    };
    auto cp4 = [&](unsigned char* dst, const float* src) {
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(dst)), "l"(src)
                   : "memory");
    };
    auto cp16 = [&](unsigned char* dst, const float* src) {
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src)
                   : "memory");
    };
    Unit x = n_units > 0 ? tile_info(t_begin) : Unit{};   // the unit copied at this step
    Unit xc = x;                                           // the unit converted at this step
    for (int64_t u = 0; u <= n_units; ++u) {
      Unit xn = x;
      if (u + 1 < n_units) xn = tile_info(t_begin + u + 1);
      const int b = (int)(u & 1);
      unsigned char* abuf = sm + kOffA + b * kABufBytes;
      // copy u: raw buffer u & 1 was last read by the conversion of unit u - 2, the slot list
      // ring's entry by the epilogue's fetch of unit u - 2
      bool ok = u >= n_units || u < 2 ||
                (wait(&bars[kBarRawFree0 + b], (uint32_t)(((u - 2) >> 1) & 1), lim, s_abort) &&
                 wait(&bars[kBarOwnFree0 + b], (uint32_t)(((u - 2) >> 1) & 1), lim, s_abort));
      if (u < n_units && ok) {
        // half-warp h of the warp takes column p + 11 (2 i + h); lane l16 the 16-byte chunk l16
        // of the other message's row (16-byte aligned: the plan starts such rows at multiples of
        // 4 slots) and of the sums' row when that is aligned too, else four single states
        const int h = lane >> 4, l16 = lane & 15;
        int* meta_own = reinterpret_cast<int*>(sm + kOffOwn) + b * kM;
#pragma unroll
        for (int i = 0; i < kColsPerProd / 2; ++i) {
          const int j = 2 * i + h;
          const int c = p + kProdWarps * j;
          const int qy = __shfl_sync(0xffffffffu, x.qy, j);
          const int qv = __shfl_sync(0xffffffffu, x.qv, j);
          if (c < x.ncols) {
            if (l16 == 0) meta_own[c] = qy + (dir == 0 ? 0 : K);
            const float* other = a.cur + qy + (dir == 0 ? K : 0);
            const float* sums = a.vsum + qv;
            const uint32_t o = sw128(c, 4 * l16, kM);
            cp16(abuf + o, other + 4 * l16);
            if ((qv & 3) == 0) {
              cp16(abuf + kABytes + o, sums + 4 * l16);
            } else {
#pragma unroll
              for (int k4 = 0; k4 < 4; ++k4)
                cp4(abuf + kABytes + sw128(c, l16 + 16 * k4, kM), sums + l16 + 16 * k4);
            }
          }
        }
        // the raw buffer is full once every producer thread's copies have landed
        asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(
                         smem_addr(&bars[kBarRawFull0 + b]))
                     : "memory");
        bar_arrive(&bars[kBarOwnFull0 + b]);
      }
      if (u >= 1) {
        // convert u - 1: its copies have landed; TMEM operand buffer (u - 1) & 1 was last read
        // by the products of unit u - 3, the maxima slot by the epilogue of unit u - 3
        const int mb = (int)((u - 1) & 1);
        ok = ok && wait(&bars[kBarRawFull0 + mb], (uint32_t)(((u - 1) >> 1) & 1), lim, s_abort);
        ok = ok && (u < 3 || (wait(&bars[kBarMma0 + mb], (uint32_t)(((u - 3) >> 1) & 1), lim,
                                   s_abort) &&
                              wait(&bars[kBarMetaFree0 + mb], (uint32_t)(((u - 3) >> 1) & 1),
                                   lim, s_abort)));
      }
      // the producers leave together (the converting warps meet at a named barrier)
      if (!named_bar_and(1, 32 * kProdWarps, ok)) {
        asm volatile("cp.async.wait_all;" ::: "memory");
        break;
      }
      if (u >= 1) {
        const int mb = (int)((u - 1) & 1);
        unsigned char* cbuf = sm + kOffA + mb * kABufBytes;
        float* meta_m = reinterpret_cast<float*>(sm + kOffM) + mb * kM;
        if (p < kCvtWarps) {
          fence_after_sync();
          convert(cbuf, mb, xc.ncols, meta_m, &bars[kBarRawFree0 + mb]);
        } else if (p == kCvtWarps) {
          // the table maxima, times 1 - damping
          float* meta_r = reinterpret_cast<float*>(sm + kOffR) + mb * K;
          meta_r[lane] = a.omd * xc.r0;
          meta_r[lane + 32] = a.omd * xc.r1;
        }
        // the operand's TMEM writes are ordered before the MMA warp's products
        fence_before_sync();
        bar_arrive(&bars[kBarAFull0 + mb]);
        bar_arrive(&bars[kBarMetaFull0 + mb]);
      }
      xc = x;
      x = xn;
    }
  } else if (warp == kMmaWarp) {
    // ------------------------------------------------------------------ MMA issue
    if (lane == 0) {
      TileCursor cur;
      int loaded = -1;
      uint32_t tab_phase = 0;
      int64_t last_commit[2] = {-1, -1};
      for (int64_t u = 0; u < n_units; ++u) {
        const int s = (int)(u & 1);
        cur.seek(a, (int)(t_begin + u));
        if (cur.g != loaded) {
          // the old tables' last reader is the previous unit's products
          if (u >= 1 && !wait(&bars[kBarMma0 + ((u - 1) & 1)], (uint32_t)(((u - 1) >> 1) & 1),
                              lim, s_abort))
            break;
          bulk_load(sm, tab_g0 + (int64_t)cur.g * kTabFloats + (int64_t)dir * 2 * K * K,
                    (uint32_t)kTabBytes, &bars[kBarTab], a.skip_copy != 0);
          if (!wait(&bars[kBarTab], tab_phase, lim, s_abort)) break;
          tab_phase ^= 1u;
          loaded = cur.g;
        }
        if (!wait(&bars[kBarAFull0 + s], (uint32_t)((u >> 1) & 1), lim, s_abort)) break;
        if (u >= 2 && !wait(&bars[kBarTmem0 + s], (uint32_t)(((u - 2) >> 1) & 1), lim, s_abort))
          break;
        fence_after_sync();
        const uint32_t d_tmem = tmem + (uint32_t)(s * K);
        const uint32_t b_hi = s_base, b_lo = s_base + (uint32_t)kMatBytes;
        const uint32_t a_hi = tmem + kTmemA + (uint32_t)(s * 128), a_lo = a_hi + 64u;
#pragma unroll
        for (int ks = 0; ks < K / 8; ++ks) {
          const uint64_t bh = kstep_desc(b_hi, ks, K), bl = kstep_desc(b_lo, ks, K);
          mma_tf32_ts(d_tmem, a_hi + 8u * ks, bh, ks > 0 ? 1u : 0u);
          mma_tf32_ts(d_tmem, a_hi + 8u * ks, bl, 1u);
          mma_tf32_ts(d_tmem, a_lo + 8u * ks, bh, 1u);
        }
        mma_commit(&bars[kBarMma0 + s]);
        last_commit[s] = u;
      }
      if (*s_abort) {
        // products committed but never waited for by the epilogue may still be running: wait
        // (bounded, apart from the abort flag) for the last commit of each accumulator stage
        // before the columns are freed
        for (int st = 0; st < 2; ++st)
          if (last_commit[st] >= 0)
            wait(&bars[kBarMma0 + st], (uint32_t)((last_commit[st] >> 1) & 1), lim, s_drain);
      }
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------------ epilogue
    // warp w takes TMEM lane quadrant qd = w % 4 (columns 32 qd .. 32 qd + 31 of the tile, thread
    // = column e) and states 32 eh .. 32 eh + 31, eh = w / 4; the two warps of a quadrant swap
    // their half-row maxima through TMEM. Rows are fetched and stored a quarter-warp per row half.
    const int qd = warp & 3, eh = warp >> 2;
    const int e = 32 * qd + lane;
    const int l8 = lane & 7, r4 = lane >> 3;
    const uint32_t lane_base = (uint32_t)(32 * qd) << 16;
    const float atl2 = a.omd * a.t * 0.693147180559945309f;
    float* stg0 = reinterpret_cast<float*>(sm + kOffStg);
    TileCursor fcur;
    struct EUnit {
      int own, ncols, c0, g;  // own: the lane's column's slot, -1 when the wait gave up
    };
    // the old messages (this warp's state half) of unit f's rows into staging buffer f & 1, at
    // the slots the producers listed
    auto fetch = [&](int64_t f) {
      EUnit x;
      const int tile = (int)(t_begin + f);
      fcur.seek(a, tile);
      x.ncols = fcur.ncols(tile);
      x.c0 = fcur.c0(tile);
      x.g = fcur.g;
      const int fs = (int)(f & 1);
      const bool ok = wait(&bars[kBarOwnFull0 + fs], (uint32_t)((f >> 1) & 1), lim, s_abort, 32);
      x.own = -1;
      if (!__all_sync(0xffffffffu, ok)) return x;
      x.own = e < x.ncols ? reinterpret_cast<const int*>(sm + kOffOwn)[fs * kM + e] : 0;
      bar_arrive(&bars[kBarOwnFree0 + fs]);
      float* stg = stg0 + fs * (kM * K);
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int r = 4 * i + r4, c = 32 * qd + r;
        const int ow = __shfl_sync(0xffffffffu, x.own, r);
        const int q = 8 * eh + l8;
        if (c < x.ncols) {
          asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                           smem_addr(stg + stg_chunk(c, q))),
                       "l"(a.cur + ow + 4 * q)
                       : "memory");
        }
      }
      asm volatile("cp.async.commit_group;" ::: "memory");
      return x;
    };
    unsigned res = 0u;
    EUnit nx = n_units > 0 ? fetch(0) : EUnit{-1, 0, 0, 0};
    for (int64_t u = 0; u < n_units; ++u) {
      const int s = (int)(u & 1);
      const int own = nx.own, ncols = nx.ncols, g = nx.g;
      const int64_t c0 = nx.c0;
      bool ok = own >= 0;
      if (u + 1 < n_units) {
        if (ok) {
          nx = fetch(u + 1);
          ok = nx.own >= 0;
        }
      } else {
        asm volatile("cp.async.commit_group;" ::: "memory");
      }
      const uint32_t ph = (uint32_t)((u >> 1) & 1);
      ok = ok && wait(&bars[kBarMetaFull0 + s], ph, lim, s_abort, 32);
      ok = ok && wait(&bars[kBarMma0 + s], ph, lim, s_abort, 32);
      ok = __all_sync(0xffffffffu, ok);   // tcgen05.ld below is warp-wide
      asm volatile("cp.async.wait_group 1;" ::: "memory");   // this unit's old messages
      __syncwarp();
      fence_after_sync();
      float* stg = stg0 + s * (kM * K);
      float* row = stg + e * K;
      const int key = e & 7;
      const float mo = a.omd * reinterpret_cast<const float*>(sm + kOffM)[s * kM + e];
      const float* rr = reinterpret_cast<const float*>(sm + kOffR) + s * K + 32 * eh;
      const bool active = e < ncols;
      // the 32 sums of the half row in one batch of TMEM loads, turned into y in place (after a
      // failed wait the values are garbage and unused: the CTA stops at the barrier below)
      uint32_t raw[2][16];
      const uint32_t tacc = tmem + lane_base + (uint32_t)(s * K + 32 * eh);
      tmem_ld16_nowait(tacc, raw[0]);
      tmem_ld16_nowait(tacc + 16u, raw[1]);
      // the first half's old messages and maxima load while the TMEM loads are in flight
      float4 o4[4], rm4[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        o4[q] = *reinterpret_cast<const float4*>(row + (((8 * eh + q) ^ key) << 2));
        rm4[q] = *reinterpret_cast<const float4*>(rr + 4 * q);
      }
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      float y[32];
#pragma unroll
      for (int k = 0; k < 32; ++k) y[k] = __uint_as_float(raw[k >> 4][k & 15]);
      float x4[4] = {-INFINITY, -INFINITY, -INFINITY, -INFINITY};
      float amin = INFINITY;   // the smallest sum (NaN if any is not a number)
#pragma unroll
      for (int h2 = 0; h2 < 2; ++h2) {
        if (h2 == 1) {
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            o4[q] = *reinterpret_cast<const float4*>(row + (((8 * eh + 4 + q) ^ key) << 2));
            rm4[q] = *reinterpret_cast<const float4*>(rr + 16 + 4 * q);
          }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float ov[4] = {o4[q].x, o4[q].y, o4[q].z, o4[q].w};
          const float rv[4] = {rm4[q].x, rm4[q].y, rm4[q].z, rm4[q].w};
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int j = 16 * h2 + 4 * q + k;
            amin = minn(amin, y[j]);
            y[j] = epi_message(a, atl2, y[j], mo + rv[k], ov[k]);
          }
        }
      }
      if (__any_sync(0xffffffffu, active && !(amin >= 1e-30f))) {
        // rare: a table row spanning more than about 69 T underflowed somewhere in the warp;
        // those states take the reference's formula
        const int4 qr = active ? a.rec[a.grp_first[g] + c0 + e] : make_int4(0, 0, 0, 0);
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const float sum = tmem_ld1(tacc + (uint32_t)j);
          if (active && !(sum >= 1e-30f)) {
            const int st = 32 * eh + j;
            y[j] = epi_message_slow(a, qr, st, dir == 0, a.grp_table[g],
                                    row[(((st >> 2) ^ key) << 2) + (st & 3)]);
          }
        }
      }
#pragma unroll
      for (int j = 0; j < 32; ++j) x4[j & 3] = maxn(x4[j & 3], y[j]);
      const float xh = maxn(maxn(x4[0], x4[1]), maxn(x4[2], x4[3]));
      // swap the half-row maxima with the other warp of the quadrant (barrier 3 + quadrant, the
      // two warps); they leave together here (the barrier ends the unit's waits); a pair that
      // stops leaves the others' waits for its arrivals to run out and stop them too
      tmem_st1(tmem + lane_base + kTmemX + (uint32_t)(2 * s + eh), __float_as_uint(xh));
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      fence_before_sync();
      if (!named_bar_and(3 + qd, 64, ok)) {
        asm volatile("cp.async.wait_all;" ::: "memory");
        break;
      }
      fence_after_sync();
      const float x = maxn(xh, __uint_as_float([&] {
        uint32_t r;
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];"
                     : "=r"(r)
                     : "r"(tmem + lane_base + kTmemX + (uint32_t)(2 * s + (eh ^ 1))));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        return r;
      }()));
      fence_before_sync();
      bar_arrive(&bars[kBarTmem0 + s]);
      bar_arrive(&bars[kBarMetaFree0 + s]);
      float dmax = 0.0f;
      if (active) {
#pragma unroll
        for (int q4 = 0; q4 < 2; ++q4) {
          float4 o[4];
#pragma unroll
          for (int k = 0; k < 4; ++k)
            o[k] = *reinterpret_cast<const float4*>(row + (((8 * eh + 4 * q4 + k) ^ key) << 2));
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int j = 16 * q4 + 4 * k;
            float4 nv;
            nv.x = maxn(y[j + 0] - x, kMsgNegInf);
            nv.y = maxn(y[j + 1] - x, kMsgNegInf);
            nv.z = maxn(y[j + 2] - x, kMsgNegInf);
            nv.w = maxn(y[j + 3] - x, kMsgNegInf);
            dmax = maxn(dmax, fabsf(nv.x - o[k].x));
            dmax = maxn(dmax, fabsf(nv.y - o[k].y));
            dmax = maxn(dmax, fabsf(nv.z - o[k].z));
            dmax = maxn(dmax, fabsf(nv.w - o[k].w));
            *reinterpret_cast<float4*>(row + (((8 * eh + 4 * q4 + k) ^ key) << 2)) = nv;
          }
        }
      }
      __syncwarp();
      // the new half rows to their slots, a quarter-warp per row, 16-byte stores
      {
        float4 v[8];
        const int q = 8 * eh + l8;
#pragma unroll
        for (int i = 0; i < 8; ++i)
          v[i] = *reinterpret_cast<const float4*>(stg + stg_chunk(32 * qd + 4 * i + r4, q));
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int r = 4 * i + r4, c = 32 * qd + r;
          const int ow = __shfl_sync(0xffffffffu, own, r);
          if (c < ncols) *reinterpret_cast<float4*>(a.nxt + ow + 4 * q) = v[i];
        }
      }
      __syncwarp();   // the rows are read before the next fetch into this buffer
      res = __float_as_uint(maxn(__uint_as_float(res), dmax));
    }
    res = __float_as_uint(warp_max(__uint_as_float(res)));
    if (lane == 0 && res != 0u) atomicMax(s_res, res);
  }

  // ---------------------------------------------------------------- teardown
  fence_before_sync();
  __syncthreads();
  if (warp == kMmaWarp) {
    fence_after_sync();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols)
                 : "memory");
  }
  if (threadIdx.x == 0) {
    if (*s_abort) {
      atomicAdd(&g_wait_timeouts, 1ull);
      if (a.fault != nullptr) {
        *reinterpret_cast<volatile unsigned*>(a.fault) = 1u;
        __threadfence_system();
      }
    } else if (a.dacc != nullptr && *s_res != 0u) {
      atomicMax(a.dacc, *s_res);
    }
  }
}

}  // namespace tc

// One iteration of a K = 64 bucket at B = 1 on the tcgen05 path: pairs of CTAs (one per SM),
// each pair over a contiguous range of 128-column tiles, one CTA per message direction.
cudaError_t launch_tc(const Plan& p, const PairwiseBucket& q, cudaStream_t s, const ExpArgs& base,
                      const float* tc_tables) {
  static const cudaError_t attr = cudaFuncSetAttribute(
      tc::pairwise_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::kSmemBytes);
  if (attr != cudaSuccess) return attr;
  ExpArgs a = base;
  int64_t tiles = 0;
  for (int64_t c : q.grp_count_host) tiles += (c + tc::kM - 1) / tc::kM;
  if (tiles == 0) return cudaSuccess;
  const int64_t ranges = std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)p.sm_count / 2));
  a.n_tiles = tiles;
  a.tiles_per_cta = (tiles + ranges - 1) / ranges;
  const int64_t grid = 2 * ((tiles + a.tiles_per_cta - 1) / a.tiles_per_cta);
  tc::pairwise_kernel<<<(unsigned)grid, tc::kThreads, tc::kSmemBytes, s>>>(a, tc_tables);
  return cudaGetLastError();
}

}  // namespace

bool expgemm_eligible(const PairwiseBucket& q) { return q.n_groups > 0; }

cudaError_t read_wait_timeouts(unsigned long long* count) {
  unsigned long long zero = 0;
  cudaError_t e = cudaMemcpyFromSymbol(count, g_wait_timeouts, sizeof(*count));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_wait_timeouts, &zero, sizeof(zero));
  return e;
}

int64_t expgemm_tc_table_floats(int K) { return K == tc::K ? tc::kTabFloats : 0; }

cudaError_t expgemm_prepare(const Plan& p, const PairwiseBucket& q, cudaStream_t s,
                            const float* lpc, float t, float* tables) {
  (void)p;
  if (q.n_groups == 0) return cudaSuccess;
  ProfileScope ps(kProfLayout, s);
  switch (q.n1) {
    case 16: expgemm_tables_kernel<16><<<q.n_groups, kThreads, 0, s>>>(q.grp_table, lpc, t, tables); break;
    case 32: expgemm_tables_kernel<32><<<q.n_groups, kThreads, 0, s>>>(q.grp_table, lpc, t, tables); break;
    case 64:
      expgemm_tables_kernel<64><<<q.n_groups, kThreads, 0, s>>>(q.grp_table, lpc, t, tables);
      // the tcgen05 path's tables follow the n_groups blocks of the layout above
      tc::tables_kernel<<<q.n_groups, 256, 0, s>>>(
          q.grp_table, lpc, t, tables + (int64_t)q.n_groups * expgemm_table_floats(64));
      break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t expgemm_iterate(const Plan& p, const PairwiseBucket& q, cudaStream_t s, int64_t B,
                            const float* cur, float* nxt, const float* vsum, const float* lpc,
                            const float* tables, float d, float omd, float t, unsigned* dacc) {
  ExpArgs a{};
  a.rec = q.rec;
  a.grp_first = q.grp_first;
  a.grp_count = q.grp_count;
  a.grp_table = q.grp_table;
  a.n_groups = q.n_groups;
  a.B = B;
  a.cur = cur;
  a.nxt = nxt;
  a.vsum = vsum;
  a.lpc = lpc;
  a.tables = tables;
  a.d = d;
  a.omd = omd;
  a.t = t;
  a.dacc = dacc;
  const DebugKnobs knobs = debug_knobs();
  a.fault = p.fault_dev;
  a.wait_ns = knobs.wait_limit_ns != 0 ? knobs.wait_limit_ns : kWaitLimitNs;
  a.skip_copy = knobs.skip_table_copy;
  // the tcgen05 kernel moves message rows as 16-byte chunks: every row and buffer aligned
  const bool aligned16 =
      q.rows16 && ((reinterpret_cast<uintptr_t>(cur) | reinterpret_cast<uintptr_t>(nxt) |
                    reinterpret_cast<uintptr_t>(vsum)) & 15u) == 0;
  // its tile cursor counts tiles and columns in int32
  const bool small = q.count + (int64_t)q.n_groups * tc::kM < (int64_t)INT32_MAX;
  if (q.n1 == 64 && B == 1 && aligned16 && small && !knobs.legacy_mma) {
    ProfileScope ps(kProfPairwiseExp, s);
    return launch_tc(p, q, s, a, tables + (int64_t)q.n_groups * expgemm_table_floats(64));
  }
  ProfileScope ps(kProfPairwise, s);
  switch (q.n1) {
    case 16: return launch<16>(p, q, s, a);
    case 32: return launch<32>(p, q, s, a);
    case 64: return launch<64>(p, q, s, a);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace pgbp
