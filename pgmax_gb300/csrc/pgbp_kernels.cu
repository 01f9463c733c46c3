// sm_103a kernels of the loopy-BP engine.
//
// Layout in HBM during a run: messages live in "slots" (pgbp_internal.h), variable sums, evidence
// and batched potentials likewise, all "slot-major, batch innermost" - element (slot s, instance
// b) at s * B + b - so the 32 lanes of a warp read 32 instances of one slot in one 128-byte
// transaction and every index is one broadcast load per warp. An edge of a binary variable owns
// a single slot: after normalize_and_clip_msgs (pgmax/infer/bp.py:222-260) one of its two states
// is exactly +0 (x - x), so the pair is stored as one float and decoded exactly (encode2/decode2
// below); this halves the message traffic of binary graphs without changing a single bit of the
// arithmetic. The caller's BPArrays are [B, n] (jax.vmap layout); run() transposes them in and out
// through shared-memory tiles.
//
// One BP iteration (pgmax/infer/bp.py:98-137) is:
//   varsum kernels   var_sums[vs] = evidence[vs] + sum of msgs over vs's edge states, serially in
//                    increasing edge-state order, the order of the reference's scatter-add
//                    (bp.py:217);
//   factor kernels   one per factor class (dense pairwise Enum, generic Enum, OR, AND, Pool). Each
//                    thread owns one (factor, instance): it forms vtof = var_sums - msgs
//                    (bp.py:218) for the factor's edges, computes the factor-to-variable messages,
//                    and applies damping, per-edge max-normalisation, clipping at MSG_NEG_INF and
//                    the residual (bp.py:127-136) before writing - a factor owns all states of its
//                    edges, so the epilogue needs nothing from other threads.
// Everything is float32 in the reference's operation order; the build uses -fmad=false so no
// multiply-add is contracted. At temperature 0 the engine reproduces the oracle bit for bit; at
// temperature > 0 expf/logf/log1pf/expm1f differ from glibc's by an ulp or two.
#include <cooperative_groups.h>
#include <math.h>

#include <algorithm>
#include <type_traits>

#include "pgbp_gumbel.h"
#include "pgbp_internal.h"

namespace pgbp {
namespace {

constexpr float kMsgNegInf = -1e32f;    // MSG_NEG_INF, pgmax/utils/__init__.py:26
constexpr float kLpMaxAbs = 1e6f;       // LOG_POTENTIAL_MAX_ABS, pgmax/utils/__init__.py:32
constexpr double kStabilityThre = 0.5;  // TEMPERATURE_STABILITY_THRE, pgmax/factor/logical.py:33

// NaN-propagating maximum / minimum, as jnp.maximum / jnp.minimum: one max.NaN / min.NaN
// instruction. It equals the reference's result for every input, up to the sign of a zero when
// +0 and -0 meet (IEEE-equal values).
__device__ __forceinline__ float fmaxp(float a, float b) {
  float r;
  asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float fminp(float a, float b) {
  float r;
  asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}

// x / t for a temperature t > 0. When t is a power of two (1, 0.5, 2, ...) its reciprocal is
// exact, so x * (1 / t) is the same correctly rounded value as x / t and costs one multiply
// instead of a full division; the reciprocal's exponent field is 254 - t's.
__device__ __forceinline__ float div_t(float x, float t) {
  const unsigned u = __float_as_uint(t);
  const unsigned e = (u >> 23) & 0xffu;
  if ((u & 0x807fffffu) == 0u && e >= 2u && e <= 252u) return x * __uint_as_float((254u - e) << 23);
  return x / t;
}

// update_utils.py:150-166
__device__ __forceinline__ float logaddexp_t(float a, float b, float t) {
  const float mx = fmaxp(a, b);
  const float mn = fminp(a, b);
  const float w = log1pf(expf(div_t(mn - mx, t)));
  return t * w + mx;
}

// update_utils.py:134-147 (both branches evaluated, as jnp.where does)
__device__ __forceinline__ float log1mexp_f(float x) {
  const float a = logf(-expm1f(-x));
  const float b = log1pf(-expf(-x));
  return (x <= 0.693147182464599609375f) ? a : b;  // float32(log(2))
}

// update_utils.py:169-190
__device__ __forceinline__ float logminusexp_t(float a, float b, float t, float eps) {
  const float v = t * log1mexp_f(div_t(a - b, t)) + a;
  return (a >= b + eps) ? v : -INFINITY;
}

// A normalised binary message (m0, m1) has m0 == 0 or m1 == 0 (or both NaN, since the
// normalising max propagates NaN to both states), so it is stored as the single float
// c = m1 - m0 (= m1 <= 0 or -m0 > 0; exact, as one operand is zero) and recovered as
// m0 = min(-c, 0), m1 = min(c, 0), with NaN staying NaN: the same values, one instruction each.
__device__ __forceinline__ float encode2(float m0, float m1) { return m1 - m0; }
__device__ __forceinline__ void decode2(float c, float& m0, float& m1) {
  m0 = fminp(-c, 0.0f);
  m1 = fminp(c, 0.0f);
}

// ----------------------------------------------------------------------------- launch mapping
// Blocks are (bx lanes over instances) x (by lanes over units); each thread keeps its instance and
// strides over units, so its residual stays in a register until one reduction per block.

struct Lane {
  int64_t b;
  bool valid;
  int64_t u0, ustep;
};

__device__ __forceinline__ Lane lane(int64_t B) {
  Lane l;
  l.b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  l.valid = l.b < B;
  l.u0 = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  l.ustep = (int64_t)gridDim.y * blockDim.y;
  return l;
}

// Max-reduces v over the block's unit lanes and folds it into dst[b] (float bits; v >= 0 or NaN,
// so unsigned order is float order and a NaN residual wins, as jnp.max propagates it).
__device__ __forceinline__ void block_max_to(unsigned* dst, const Lane& l, float v) {
  __shared__ float red[256];
  const int tx = threadIdx.x, ty = threadIdx.y, bx = blockDim.x;
  red[ty * bx + tx] = v;
  __syncthreads();
  for (int s = blockDim.y / 2; s > 0; s >>= 1) {
    if (ty < s) red[ty * bx + tx] = fmaxp(red[ty * bx + tx], red[(ty + s) * bx + tx]);
    __syncthreads();
  }
  if (ty == 0 && l.valid && dst != nullptr) atomicMax(dst + l.b, __float_as_uint(red[tx]));
}

// ----------------------------------------------------------------------------- contexts
// An edge seen by a factor: its first edge state (caller layout), its first slot (run layout) and
// its variable's first state (variable sums).
struct EdgeRef {
  int64_t es0, slot, vs0;
};

__device__ __forceinline__ EdgeRef edge_ref(int4 r) { return EdgeRef{r.x, r.y, r.z}; }

// Fused: inside run(). vtof from variable sums and the current messages; outputs go through
// damping, normalisation, clipping and the residual into the next messages.
struct Fused {
  const float* __restrict__ cur;
  float* __restrict__ nxt;
  const float* __restrict__ vsum;
  const float* __restrict__ lp;
  int64_t lps, lpb;  // potential k of instance b at lp[k * lps + b * lpb]
  int64_t B;
  float d, omd;

  __device__ __forceinline__ float pot(int64_t k, int64_t b) const {
    return __ldg(lp + k * lps + b * lpb);
  }

  // old[i] = current message, vt[i] = variable-to-factor message of the edge's k states.
  __device__ __forceinline__ void load(const EdgeRef& r, int k, int64_t b, float* old,
                                       float* vt) const {
    if (k == 2) {
      decode2(cur[r.slot * B + b], old[0], old[1]);
    } else {
      for (int i = 0; i < k; ++i) old[i] = cur[(r.slot + i) * B + b];
    }
    for (int i = 0; i < k; ++i) vt[i] = vsum[(r.vs0 + i) * B + b] - old[i];
  }
  // State i of what load gives, one state at a time.
  __device__ __forceinline__ float old_at(const EdgeRef& r, int k, int i, int64_t b) const {
    if (k == 2) {
      float o0, o1;
      decode2(cur[r.slot * B + b], o0, o1);
      return i == 0 ? o0 : o1;
    }
    return cur[(r.slot + i) * B + b];
  }
  __device__ __forceinline__ float vt_at(const EdgeRef& r, int k, int i, int64_t b) const {
    return vsum[(r.vs0 + i) * B + b] - old_at(r, k, i, b);
  }

  // bp.py:127-136 for one edge; outv(i) is the new factor-to-variable message of state i, old[i]
  // the current one (an array or an accessor).
  template <class O, class F>
  __device__ __forceinline__ void store(const EdgeRef& r, int k, const O& old, F outv,
                                        int64_t b, float& dmax) const {
    if (k == 2) {
      const float n0 = d * old[0] + omd * outv(0);
      const float n1 = d * old[1] + omd * outv(1);
      const float m = fmaxp(n0, n1);  // = max(max(-inf, n0), n1) for every input
      const float v0 = fmaxp(n0 - m, kMsgNegInf);
      const float v1 = fmaxp(n1 - m, kMsgNegInf);
      nxt[r.slot * B + b] = encode2(v0, v1);
      dmax = fmaxp(dmax, fabsf(v0 - old[0]));
      dmax = fmaxp(dmax, fabsf(v1 - old[1]));
      return;
    }
    float m = -INFINITY;
#pragma unroll
    for (int i = 0; i < k; ++i) m = fmaxp(m, d * old[i] + omd * outv(i));
#pragma unroll
    for (int i = 0; i < k; ++i) {
      const float n = d * old[i] + omd * outv(i);
      const float v = fmaxp(n - m, kMsgNegInf);
      nxt[(r.slot + i) * B + b] = v;
      dmax = fmaxp(dmax, fabsf(v - old[i]));
    }
  }
};

// Minimum resident blocks of 256 threads per SM the dense 2 x 2 pairwise kernel is compiled for,
// per access class (the register budget follows: 65536 / (256 * blocks)).
template <class C>
struct PairwiseMinBlocks {
  static constexpr int value = 1;
};

// Update: one factor type's raw update on caller arrays [B, n_type] (a FAC_TO_VAR_UPDATES call).
struct Update {
  const float* __restrict__ vt;
  int64_t vts;
  float* __restrict__ out;
  int64_t os;
  int64_t base;  // first edge state of the type
  const float* __restrict__ lp;
  int64_t lpb;   // instance stride of the potentials (0 = shared)
  int64_t lpbase;

  __device__ __forceinline__ float pot(int64_t k, int64_t b) const {
    return lp[b * lpb + (k - lpbase)];
  }
  __device__ __forceinline__ void load(const EdgeRef& r, int k, int64_t b, float* old,
                                       float* vtof) const {
    for (int i = 0; i < k; ++i) {
      old[i] = 0.0f;
      vtof[i] = vt[b * vts + (r.es0 + i - base)];
    }
  }
  __device__ __forceinline__ float old_at(const EdgeRef&, int, int, int64_t) const { return 0.0f; }
  __device__ __forceinline__ float vt_at(const EdgeRef& r, int, int i, int64_t b) const {
    return vt[b * vts + (r.es0 + i - base)];
  }
  template <class O, class F>
  __device__ __forceinline__ void store(const EdgeRef& r, int k, const O&, F outv, int64_t b,
                                        float&) const {
    for (int i = 0; i < k; ++i) out[b * os + (r.es0 + i - base)] = outv(i);
  }
};

// ----------------------------------------------------------------------------- Enum factors
// pass_enum_fac_to_var_messages, pgmax/factor/enum.py:451-475, for one dense pairwise factor.
// summary(i, j) = ((0 + vtof1[i]) + vtof2[j]) + lp[i * n2 + j]; the max / sum-exp over the configs
// of an edge state run in increasing config order, the reference's scatter order.
template <int N1, int N2, bool T0, class C>
__device__ __forceinline__ void pairwise_body(const C& c, const EdgeRef& r1, const EdgeRef& r2,
                                              int64_t k0, int n1d, int n2d, int64_t b, float t,
                                              float& dmax) {
  // N1, N2 > 0: sizes known at compile time, arrays live in registers (loops unroll).
  // N1 = N2 = 0: run-time sizes up to 64, arrays in local memory.
  constexpr int M1 = N1 > 0 ? N1 : 64;
  constexpr int M2 = N2 > 0 ? N2 : 64;
  const int n1 = N1 > 0 ? N1 : n1d;
  const int n2 = N2 > 0 ? N2 : n2d;
  float o1[M1], o2[M2], v1[M1], v2[M2], mx1[M1], mx2[M2];
  c.load(r1, n1, b, o1, v1);
  c.load(r2, n2, b, o2, v2);
  for (int i = 0; i < n1; ++i) mx1[i] = -INFINITY;
  for (int j = 0; j < n2; ++j) mx2[j] = -INFINITY;
  for (int i = 0; i < n1; ++i) {
    for (int j = 0; j < n2; ++j) {
      const float s = ((0.0f + v1[i]) + v2[j]) + c.pot(k0 + i * n2 + j, b);
      mx1[i] = fmaxp(mx1[i], s);
      mx2[j] = fmaxp(mx2[j], s);
    }
  }
  if (T0) {
    c.store(r1, n1, o1, [&](int i) { return mx1[i] - v1[i]; }, b, dmax);
    c.store(r2, n2, o2, [&](int j) { return mx2[j] - v2[j]; }, b, dmax);
  } else {
    float s1[M1], s2[M2];
    for (int i = 0; i < n1; ++i) s1[i] = 0.0f;
    for (int j = 0; j < n2; ++j) s2[j] = 0.0f;
    for (int i = 0; i < n1; ++i) {
      for (int j = 0; j < n2; ++j) {
        const float s = ((0.0f + v1[i]) + v2[j]) + c.pot(k0 + i * n2 + j, b);
        s1[i] += expf(div_t(s - mx1[i], t));
        s2[j] += expf(div_t(s - mx2[j], t));
      }
    }
    c.store(r1, n1, o1, [&](int i) { return (t * logf(s1[i]) + mx1[i]) - v1[i]; }, b, dmax);
    c.store(r2, n2, o2, [&](int j) { return (t * logf(s2[j]) + mx2[j]) - v2[j]; }, b, dmax);
  }
}

struct PairwiseDev {
  const int4* __restrict__ rec;
  const int32_t* __restrict__ cfg_begin;
  int64_t count;
  int n1, n2;
};

__device__ __forceinline__ void pairwise_refs(const PairwiseDev& p, int4 q, EdgeRef& r1,
                                              EdgeRef& r2) {
  r1 = EdgeRef{q.x, q.y, q.z};
  r2 = EdgeRef{(int64_t)q.x + p.n1, (int64_t)q.y + (p.n1 == 2 ? 1 : p.n1), q.w};
}

template <int N1, int N2, bool T0, class C>
__global__ void __launch_bounds__(256, (N1 == 2 && N2 == 2)   ? PairwiseMinBlocks<C>::value
                                      : (N1 == 8 && N2 == 8) ? 2
                                                             : 1)
    pairwise_kernel(C c, PairwiseDev p, int64_t B, float t, unsigned* deltas) {
  pdl_begin();
  const Lane l = lane(B);
  float dmax = 0.0f;
  // two factors per step for tables of up to 16 entries: their loads are independent, so twice
  // as many are in flight; larger tables keep one (two would double the live state)
  constexpr bool kPairs = N1 > 0 && N1 * N2 <= 16;
  if (l.valid) {
    int64_t u = l.u0;
    for (; kPairs && u + l.ustep < p.count; u += 2 * l.ustep) {
      const int4 qa = __ldg(p.rec + u);
      const int4 qb = __ldg(p.rec + u + l.ustep);
      const int64_t ka = __ldg(p.cfg_begin + u), kb = __ldg(p.cfg_begin + u + l.ustep);
      EdgeRef a1, a2, b1, b2;
      pairwise_refs(p, qa, a1, a2);
      pairwise_refs(p, qb, b1, b2);
      pairwise_body<N1, N2, T0>(c, a1, a2, ka, p.n1, p.n2, l.b, t, dmax);
      pairwise_body<N1, N2, T0>(c, b1, b2, kb, p.n1, p.n2, l.b, t, dmax);
    }
    for (; u < p.count; u += l.ustep) {
      EdgeRef a1, a2;
      pairwise_refs(p, __ldg(p.rec + u), a1, a2);
      pairwise_body<N1, N2, T0>(c, a1, a2, __ldg(p.cfg_begin + u), p.n1, p.n2, l.b, t, dmax);
    }
  }
  block_max_to(deltas, l, dmax);
}

struct EnumGenericDev {
  const int32_t* __restrict__ es_begin;
  const int32_t* __restrict__ n_es;
  const int32_t* __restrict__ edge_off;
  const int32_t* __restrict__ edge_size;
  const int32_t* __restrict__ edge_slot;
  const int32_t* __restrict__ edge_vs;
  const int32_t* __restrict__ row_begin;
  const int32_t* __restrict__ n_cfg;
  const int32_t* __restrict__ n_vars;
  const int32_t* __restrict__ cfg_begin;
  const int32_t* __restrict__ row_les;
  int64_t count;
  const int32_t* __restrict__ inv_begin;
  const int32_t* __restrict__ inv_off;
  const int32_t* __restrict__ inv_cfg;
};

// pass_enum_fac_to_var_messages (enum.py:451-475) for an arbitrary config table: factor f,
// instance b.
template <int MAXES, bool T0, class C>
__device__ __forceinline__ void enum_generic_unit(const C& c, const EnumGenericDev& g, int64_t f,
                                                  int64_t b, float t, float& dmax) {
  const int64_t e0 = g.es_begin[f];
  const int n = g.n_es[f], nv = g.n_vars[f], ncfg = g.n_cfg[f];
  const int64_t rb = g.row_begin[f], k0 = g.cfg_begin[f];
  const int j0 = g.edge_off[f], j1 = g.edge_off[f + 1];
  float old[MAXES], v[MAXES], mx[MAXES], se[MAXES];
  {
    int pos = 0;
    for (int j = j0; j < j1; ++j) {
      const int k = g.edge_size[j];
      c.load(EdgeRef{e0 + pos, g.edge_slot[j], g.edge_vs[j]}, k, b, old + pos, v + pos);
      pos += k;
    }
  }
  for (int i = 0; i < n; ++i) {
    mx[i] = -INFINITY;
    se[i] = 0.0f;
  }
  for (int k = 0; k < ncfg; ++k) {
    const int32_t* rows = g.row_les + rb + (int64_t)k * nv;
    float s = 0.0f;
    for (int i = 0; i < nv; ++i) s += v[rows[i]];
    s = s + c.pot(k0 + k, b);
    for (int i = 0; i < nv; ++i) mx[rows[i]] = fmaxp(mx[rows[i]], s);
  }
  if (!T0) {
    for (int k = 0; k < ncfg; ++k) {
      const int32_t* rows = g.row_les + rb + (int64_t)k * nv;
      float s = 0.0f;
      for (int i = 0; i < nv; ++i) s += v[rows[i]];
      s = s + c.pot(k0 + k, b);
      for (int i = 0; i < nv; ++i) se[rows[i]] += expf(div_t(s - mx[rows[i]], t));
    }
  }
  int pos = 0;
  for (int j = j0; j < j1; ++j) {
    const int k = g.edge_size[j];
    const int p0 = pos;
    const EdgeRef r{e0 + pos, g.edge_slot[j], g.edge_vs[j]};
    if (T0) {
      c.store(r, k, old + p0, [&](int i) { return mx[p0 + i] - v[p0 + i]; }, b, dmax);
    } else {
      c.store(r, k, old + p0,
              [&](int i) { return (t * logf(se[p0 + i]) + mx[p0 + i]) - v[p0 + i]; }, b, dmax);
    }
    pos += k;
  }
}

template <int MAXES, bool T0, class C>
__global__ void __launch_bounds__(256) enum_generic_kernel(C c, EnumGenericDev g, int64_t B,
                                                           float t, unsigned* deltas) {
  pdl_begin();
  const Lane l = lane(B);
  float dmax = 0.0f;
  if (l.valid) {
    for (int64_t f = l.u0; f < g.count; f += l.ustep)
      enum_generic_unit<MAXES, T0>(c, g, f, l.b, t, dmax);
  }
  block_max_to(deltas, l, dmax);
}

// The current messages of one edge, read through the context state by state (the values its
// load gives), for a store that takes them as old[i].
template <class C>
struct OldAt {
  const C& c;
  EdgeRef r;
  int k;
  int64_t b;
  __device__ __forceinline__ float operator[](int i) const { return c.old_at(r, k, i, b); }
};

// Contexts with old_at / vt_at, which the staged kernel reads edges through.
template <class C>
struct HasStaged {
  static constexpr bool value = false;
};
template <>
struct HasStaged<Fused> {
  static constexpr bool value = true;
};
template <>
struct HasStaged<Update> {
  static constexpr bool value = true;
};

// pass_enum_fac_to_var_messages (enum.py:451-475) for arbitrary config tables, staged in shared
// memory: one CTA per (factor, group of ib instances), thread (item, j) with j = instance of
// the group. Per factor, in shared memory:
//   vt_s[e][j]  the variable-to-factor message of local edge state e
//   mx_s[e][j]  the max of the config sums over the configs holding e; se_s[e][j] (T > 0) the
//               sum of exp((sum - max) / t) over them
//   rows_s      a tile of up to tk config rows (local edge states), copied from the table
//   s_s[q][j]   the config sums of the tile
// Per tile the config sums run with threads over (config, instance): the row's messages in
// variable order, then the potential. The max over each edge state's configs then runs with
// threads over (edge state, instance), along the factor's configs-by-edge-state list, whose
// position per edge state carries from tile to tile in cur_s. At T > 0 a second pass over the
// tiles sums the exponentials the same way. Each value goes through enum_generic_unit's
// operations in the same order (sums in variable order, max and exp-sum in increasing config
// order), so the two kernels give bit-identical messages.
constexpr int kStagedThreads = 256;

struct StagedShape {
  int ib, tk;
  size_t smem;
};

__host__ __device__ inline size_t staged_smem_bytes(int ib, int tk, int max_es, int max_nv, bool t0) {
  const size_t floats = (size_t)max_es * ib * (t0 ? 2 : 3) + (size_t)tk * ib + kStagedThreads;
  const size_t ints = (size_t)tk * max_nv + 2 * (size_t)max_es + (size_t)max_nv + 1;
  return 4 * (floats + ints);
}

template <bool T0, class C>
__global__ void __launch_bounds__(kStagedThreads) enum_staged_kernel(
    C c, EnumGenericDev g, int64_t B, int ib, int tk, int max_es, int max_nv, float t,
    unsigned* deltas) {
  pdl_begin();
  extern __shared__ float4 staged_smem4[];
  float* vt_s = reinterpret_cast<float*>(staged_smem4);
  float* mx_s = vt_s + max_es * ib;
  float* se_s = mx_s + max_es * ib;  // T > 0 only
  float* s_s = se_s + (T0 ? 0 : max_es * ib);
  float* red = s_s + tk * ib;
  int32_t* rows_s = reinterpret_cast<int32_t*>(red + kStagedThreads);
  int32_t* cur_s = rows_s + tk * max_nv;  // [2][max_es] list positions, by tile parity
  int32_t* pos_s = cur_s + 2 * max_es;    // [max_nv + 1] first local edge state of each edge
  const int tid = threadIdx.x;
  const int j = tid % ib, item0 = tid / ib, nitem = kStagedThreads / ib;
  const int64_t b = (int64_t)blockIdx.x * ib + j;
  const bool valid = b < B;  // instance 0 of every group is valid
  float dmax = 0.0f;
  for (int64_t f = blockIdx.y; f < g.count; f += gridDim.y) {
    const int64_t e0 = g.es_begin[f];
    const int nes = g.n_es[f], nv = g.n_vars[f], ncfg = g.n_cfg[f];
    const int64_t rb = g.row_begin[f], k0 = g.cfg_begin[f];
    const int ej0 = g.edge_off[f];
    const int32_t* io = g.inv_off + g.inv_begin[f];
    const int32_t* __restrict__ ic = g.inv_cfg;
    __syncthreads();  // the previous factor is done with the shared arrays
    if (tid == 0) {
      int pos = 0;
      for (int q = 0; q < nv; ++q) {
        pos_s[q] = pos;
        pos += g.edge_size[ej0 + q];
      }
      pos_s[nv] = pos;
    }
    __syncthreads();
    for (int q = item0; q < nv; q += nitem) {
      const int pos = pos_s[q], k = pos_s[q + 1] - pos;
      const EdgeRef r{e0 + pos, g.edge_slot[ej0 + q], g.edge_vs[ej0 + q]};
      for (int i = 0; i < k; ++i) {
        vt_s[(pos + i) * ib + j] = valid ? c.vt_at(r, k, i, b) : 0.0f;
        mx_s[(pos + i) * ib + j] = -INFINITY;
        if (!T0) se_s[(pos + i) * ib + j] = 0.0f;
      }
    }
    for (int pass = 0; pass < (T0 ? 1 : 2); ++pass) {
      __syncthreads();  // messages in place; the previous pass is done with the lists
      for (int e = tid; e < nes; e += kStagedThreads) cur_s[e] = io[e];
      int par = 0;
      for (int c0 = 0; c0 < ncfg; c0 += tk, par ^= 1) {
        const int cn = min(tk, ncfg - c0), c1 = c0 + cn;
        const bool last = c1 >= ncfg;
        __syncthreads();  // positions set; the previous tile is done with rows_s and s_s
        const int32_t* src = g.row_les + rb + (int64_t)c0 * nv;
        for (int x = tid; x < cn * nv; x += kStagedThreads) rows_s[x] = __ldg(src + x);
        __syncthreads();
        if (valid) {
          // four configs per step, their loads issued together; each sum keeps variable order
          int q = item0;
          for (; q + 3 * nitem < cn; q += 4 * nitem) {
            const int32_t* row0 = rows_s + q * nv;
            const int32_t* row1 = row0 + nitem * nv;
            const int32_t* row2 = row1 + nitem * nv;
            const int32_t* row3 = row2 + nitem * nv;
            float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
            for (int i = 0; i < nv; ++i) {
              const float x0 = vt_s[row0[i] * ib + j], x1 = vt_s[row1[i] * ib + j];
              const float x2 = vt_s[row2[i] * ib + j], x3 = vt_s[row3[i] * ib + j];
              s0 += x0;
              s1 += x1;
              s2 += x2;
              s3 += x3;
            }
            const int64_t kq = k0 + c0 + q;
            s0 = s0 + c.pot(kq, b);
            s1 = s1 + c.pot(kq + nitem, b);
            s2 = s2 + c.pot(kq + 2 * nitem, b);
            s3 = s3 + c.pot(kq + 3 * nitem, b);
            s_s[q * ib + j] = s0;
            s_s[(q + nitem) * ib + j] = s1;
            s_s[(q + 2 * nitem) * ib + j] = s2;
            s_s[(q + 3 * nitem) * ib + j] = s3;
          }
          for (; q < cn; q += nitem) {
            const int32_t* row = rows_s + q * nv;
            float sum = 0.0f;
            for (int i = 0; i < nv; ++i) sum += vt_s[row[i] * ib + j];
            sum = sum + c.pot(k0 + c0 + q, b);
            s_s[q * ib + j] = sum;
          }
        }
        __syncthreads();
        for (int e = item0; e < nes; e += nitem) {
          const int p0 = cur_s[par * max_es + e];
          int pe = io[e + 1];
          if (!last) {  // the list's configs below c1: a binary search of the sorted list
            int lo = p0, hi = pe;
            while (lo < hi) {
              const int mid = (lo + hi) >> 1;
              if (__ldg(ic + mid) < c1) lo = mid + 1;
              else hi = mid;
            }
            pe = lo;
            if (j == 0) cur_s[(par ^ 1) * max_es + e] = pe;
          }
          if (!valid) continue;
          const int x = e * ib + j;
          // eight list entries per step: their loads issued together, folded in list order
          if (pass == 0) {
            float m = mx_s[x];
            int p = p0;
            for (; p + 8 <= pe; p += 8) {
              float v[8];
#pragma unroll
              for (int u = 0; u < 8; ++u) v[u] = s_s[(__ldg(ic + p + u) - c0) * ib + j];
#pragma unroll
              for (int u = 0; u < 8; ++u) m = fmaxp(m, v[u]);
            }
            for (; p < pe; ++p) m = fmaxp(m, s_s[(__ldg(ic + p) - c0) * ib + j]);
            mx_s[x] = m;
          } else {
            const float m = mx_s[x];
            float se = se_s[x];
            int p = p0;
            for (; p + 8 <= pe; p += 8) {
              float v[8];
#pragma unroll
              for (int u = 0; u < 8; ++u) v[u] = s_s[(__ldg(ic + p + u) - c0) * ib + j];
#pragma unroll
              for (int u = 0; u < 8; ++u) v[u] = expf(div_t(v[u] - m, t));
#pragma unroll
              for (int u = 0; u < 8; ++u) se += v[u];
            }
            for (; p < pe; ++p) se += expf(div_t(s_s[(__ldg(ic + p) - c0) * ib + j] - m, t));
            se_s[x] = se;
          }
        }
      }
    }
    __syncthreads();
    if (valid) {
      for (int q = item0; q < nv; q += nitem) {
        const int pos = pos_s[q], k = pos_s[q + 1] - pos;
        const EdgeRef r{e0 + pos, g.edge_slot[ej0 + q], g.edge_vs[ej0 + q]};
        const OldAt<C> old{c, r, k, b};
        const float* vq = vt_s + pos * ib + j;
        const float* mq = mx_s + pos * ib + j;
        if (T0) {
          c.store(r, k, old, [&](int i) { return mq[i * ib] - vq[i * ib]; }, b, dmax);
        } else {
          const float* sq = se_s + pos * ib + j;
          c.store(r, k, old, [&](int i) { return (t * logf(sq[i * ib]) + mq[i * ib]) - vq[i * ib]; },
                  b, dmax);
        }
      }
    }
  }
  __syncthreads();
  red[tid] = dmax;
  __syncthreads();
  if (tid < ib && valid && deltas != nullptr) {
    float m = red[tid];
    for (int q = 1; q < nitem; ++q) m = fmaxp(m, red[q * ib + tid]);
    atomicMax(deltas + b, __float_as_uint(m));
  }
}

// ----------------------------------------------------------------------------- OR / AND factors
struct LogicalDev {
  const int32_t* __restrict__ par_begin;
  const int4* __restrict__ par;
  const int4* __restrict__ child;
  int64_t count;
  int off;
};

// (other, relevant) variable-to-factor messages of a binary edge: relevant = state 1 for OR,
// state 0 for AND; old[] receives the current messages in state order.
template <class C>
__device__ __forceinline__ void load_or(const C& c, const EdgeRef& r, int rel, int64_t b,
                                        float* old, float& v_oth, float& v_rel) {
  float vt[2];
  c.load(r, 2, b, old, vt);
  v_rel = vt[rel];
  v_oth = vt[1 - rel];
}

// pass_logical_fac_to_var_messages, pgmax/factor/logical.py:561-779: factor f, instance b.
// Factor-level sums run over the parents in order (the reference's scatter order); the argmax is
// the last parent attaining the maximum difference (update_utils.py:48-63).
template <bool T0, class C>
__device__ __forceinline__ void logical_unit(const C& c, const LogicalDev& g, int64_t f, int64_t b,
                                             float t, bool low_t, int normalize, float& dmax) {
  const int rel = g.off > 0 ? 1 : 0;
  const int64_t p0 = g.par_begin[f], p1 = g.par_begin[f + 1];
  float old[2];
  float fs_oth = 0.0f, max1 = -INFINITY, fs_x = 0.0f;
  for (int64_t i = p0; i < p1; ++i) {
    float vo, vr;
    load_or(c, edge_ref(g.par[i]), rel, b, old, vo, vr);
    fs_oth += vo;
    max1 = fmaxp(max1, vr - vo);
    fs_x += T0 ? fmaxp(vo, vr) : logaddexp_t(vr, vo, t);
  }
  int64_t arg = p1 - 1;
  {
    int64_t last = -1;
    for (int64_t i = p0; i < p1; ++i) {
      float vo, vr;
      load_or(c, edge_ref(g.par[i]), rel, b, old, vo, vr);
      if (vr - vo == max1) last = i;
    }
    if (last >= 0) arg = last;
  }
  float max2 = -INFINITY;
  for (int64_t i = p0; i < p1; ++i) {
    float vo, vr;
    load_or(c, edge_ref(g.par[i]), rel, b, old, vo, vr);
    max2 = fmaxp(max2, (i == arg) ? -INFINITY : vr - vo);
  }
  const EdgeRef rc = edge_ref(g.child[f]);
  float cold[2], c_oth, c_rel;
  load_or(c, rc, rel, b, cold, c_oth, c_rel);
  float ch_rel;
  if (T0) {
    ch_rel = fs_x + fminp(0.0f, max1);
  } else {
    ch_rel = logminusexp_t(fs_x, fs_oth, t, 1e-4f);
    if (low_t) ch_rel = fmaxp(ch_rel, logaddexp_t(fs_oth + max1, fs_oth + max2, t));
  }
  const bool single = (p1 - p0) == 1;
  for (int64_t i = p0; i < p1; ++i) {
    const EdgeRef r = edge_ref(g.par[i]);
    float vo, vr;
    load_or(c, r, rel, b, old, vo, vr);
    float p_rel, p_oth;
    if (T0) {
      const float mx = fmaxp(vo, vr);
      p_rel = (fs_x + c_rel) - mx;
      const float opt1 = (c_oth + fs_oth) - vo;
      const float opt2 = p_rel + fminp(0.0f, i == arg ? max2 : max1);
      p_oth = fmaxp(opt1, opt2);
    } else {
      const float lse = logaddexp_t(vr, vo, t);
      const float fs_lse_wo = fs_x - lse;
      const float fs_oth_wo = fs_oth - vo;
      p_rel = c_rel + fs_lse_wo;
      const float opt1 = c_oth + fs_oth_wo;
      const float opt2 = c_rel + fs_lse_wo;
      const float opt3 = c_rel + fs_oth_wo;
      p_oth = logminusexp_t(logaddexp_t(opt1, opt2, t), opt3, t, 1e-4f);
      if (low_t) {
        const float fsp = fs_oth_wo + (i == arg ? max2 : max1);
        p_oth = fmaxp(p_oth, logaddexp_t(opt1, c_rel + fsp, t));
      }
    }
    if (single) {
      p_rel = c_rel;
      p_oth = c_oth;
    }
    const float rel_out = normalize ? p_rel - p_oth : p_rel;
    const float oth_out = normalize ? 0.0f : p_oth;
    c.store(r, 2, old, [&](int s) { return s == rel ? rel_out : oth_out; }, b, dmax);
  }
  const float crel_out = normalize ? ch_rel - fs_oth : ch_rel;
  const float coth_out = normalize ? 0.0f : fs_oth;
  c.store(rc, 2, cold, [&](int s) { return s == rel ? crel_out : coth_out; }, b, dmax);
}

template <bool T0, class C>
__global__ void __launch_bounds__(256) logical_kernel(C c, LogicalDev g, int64_t B, float t,
                                                      bool low_t, int normalize, unsigned* deltas) {
  pdl_begin();
  const Lane l = lane(B);
  float dmax = 0.0f;
  if (l.valid) {
    for (int64_t f = l.u0; f < g.count; f += l.ustep)
      logical_unit<T0>(c, g, f, l.b, t, low_t, normalize, dmax);
  }
  block_max_to(deltas, l, dmax);
}

// The same update with one warp per (factor, instance), for factors with many parents: lanes
// load parents 32 at a time and compute their terms in parallel; the factor sums are accumulated
// in parent order by every lane from the shuffled terms (the same float additions in the same
// order as logical_unit, so the results are identical); maxima and the last argmax are warp
// reductions; the outputs of the parents are computed by their lanes.
__device__ __forceinline__ float warp_max(float x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = fmaxp(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}

template <bool T0, class C>
__device__ __forceinline__ void logical_warp_unit(const C& c, const LogicalDev& g, int64_t f,
                                                  int64_t b, float t, bool low_t, int normalize,
                                                  int lane, float& dmax) {
  const int rel = g.off > 0 ? 1 : 0;
  const int64_t p0 = g.par_begin[f], p1 = g.par_begin[f + 1];
  float old[2];
  float fs_oth = 0.0f, max1 = -INFINITY, fs_x = 0.0f;
  for (int64_t base = p0; base < p1; base += 32) {
    const int64_t i = base + lane;
    float vo = 0.0f, vr = 0.0f, x = 0.0f;
    if (i < p1) {
      load_or(c, edge_ref(g.par[i]), rel, b, old, vo, vr);
      x = T0 ? fmaxp(vo, vr) : logaddexp_t(vr, vo, t);
      max1 = fmaxp(max1, vr - vo);
    }
    const int n = (int)(p1 - base < 32 ? p1 - base : 32);
    for (int k = 0; k < n; ++k) {
      fs_oth += __shfl_sync(0xffffffffu, vo, k);
      fs_x += __shfl_sync(0xffffffffu, x, k);
    }
  }
  max1 = warp_max(max1);
  // the last parent attaining the maximum difference
  int64_t last = -1;
  for (int64_t i = p0 + lane; i < p1; i += 32) {
    float vo, vr;
    load_or(c, edge_ref(g.par[i]), rel, b, old, vo, vr);
    if (vr - vo == max1) last = i;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const long long other = __shfl_xor_sync(0xffffffffu, (long long)last, o);
    last = other > last ? other : last;
  }
  const int64_t arg = last >= 0 ? last : p1 - 1;
  float max2 = -INFINITY;
  for (int64_t i = p0 + lane; i < p1; i += 32) {
    float vo, vr;
    load_or(c, edge_ref(g.par[i]), rel, b, old, vo, vr);
    max2 = fmaxp(max2, (i == arg) ? -INFINITY : vr - vo);
  }
  max2 = warp_max(max2);
  const EdgeRef rc = edge_ref(g.child[f]);
  float cold[2], c_oth, c_rel;
  load_or(c, rc, rel, b, cold, c_oth, c_rel);
  float ch_rel;
  if (T0) {
    ch_rel = fs_x + fminp(0.0f, max1);
  } else {
    ch_rel = logminusexp_t(fs_x, fs_oth, t, 1e-4f);
    if (low_t) ch_rel = fmaxp(ch_rel, logaddexp_t(fs_oth + max1, fs_oth + max2, t));
  }
  const bool single = (p1 - p0) == 1;
  for (int64_t i = p0 + lane; i < p1; i += 32) {
    const EdgeRef r = edge_ref(g.par[i]);
    float vo, vr;
    load_or(c, r, rel, b, old, vo, vr);
    float p_rel, p_oth;
    if (T0) {
      const float mx = fmaxp(vo, vr);
      p_rel = (fs_x + c_rel) - mx;
      const float opt1 = (c_oth + fs_oth) - vo;
      const float opt2 = p_rel + fminp(0.0f, i == arg ? max2 : max1);
      p_oth = fmaxp(opt1, opt2);
    } else {
      const float lse = logaddexp_t(vr, vo, t);
      const float fs_lse_wo = fs_x - lse;
      const float fs_oth_wo = fs_oth - vo;
      p_rel = c_rel + fs_lse_wo;
      const float opt1 = c_oth + fs_oth_wo;
      const float opt2 = c_rel + fs_lse_wo;
      const float opt3 = c_rel + fs_oth_wo;
      p_oth = logminusexp_t(logaddexp_t(opt1, opt2, t), opt3, t, 1e-4f);
      if (low_t) {
        const float fsp = fs_oth_wo + (i == arg ? max2 : max1);
        p_oth = fmaxp(p_oth, logaddexp_t(opt1, c_rel + fsp, t));
      }
    }
    if (single) {
      p_rel = c_rel;
      p_oth = c_oth;
    }
    const float rel_out = normalize ? p_rel - p_oth : p_rel;
    const float oth_out = normalize ? 0.0f : p_oth;
    c.store(r, 2, old, [&](int s) { return s == rel ? rel_out : oth_out; }, b, dmax);
  }
  if (lane == 0) {
    const float crel_out = normalize ? ch_rel - fs_oth : ch_rel;
    const float coth_out = normalize ? 0.0f : fs_oth;
    c.store(rc, 2, cold, [&](int s) { return s == rel ? crel_out : coth_out; }, b, dmax);
  }
}

// One warp per (factor, instance) unit, unit = factor * B + instance; the residual is folded per
// block when the batch has one instance, else per warp.
template <bool T0, class C>
__global__ void __launch_bounds__(256) logical_warp_kernel(C c, LogicalDev g, int64_t B, float t,
                                                           bool low_t, int normalize,
                                                           unsigned* deltas) {
  pdl_begin();
  const int lane = threadIdx.x & 31;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t wstep = ((int64_t)gridDim.x * blockDim.x) >> 5;
  float dmax = 0.0f;
  for (int64_t u = w0; u < g.count * B; u += wstep) {
    const int64_t f = u / B, b = u % B;
    float dm = 0.0f;
    logical_warp_unit<T0>(c, g, f, b, t, low_t, normalize, lane, dm);
    dm = warp_max(dm);
    if (B == 1) {
      dmax = fmaxp(dmax, dm);
    } else if (lane == 0 && deltas != nullptr) {
      atomicMax(deltas + b, __float_as_uint(dm));
    }
  }
  if (B == 1) {
    __shared__ float red[8];
    if (lane == 0) red[threadIdx.x >> 5] = dmax;
    __syncthreads();
    if (threadIdx.x == 0 && deltas != nullptr) {
      float m = 0.0f;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmaxp(m, red[w]);
      atomicMax(deltas, __float_as_uint(m));
    }
  }
}

// ----------------------------------------------------------------------------- Pool factors
struct PoolDev {
  const int32_t* __restrict__ ch_begin;
  const int4* __restrict__ ch;
  const int4* __restrict__ ind;
  int64_t count;
};

// pass_pool_fac_to_var_messages, pgmax/factor/pool.py:328-474 (state 1 is the "on" state):
// factor f, instance b.
template <bool T0, class C>
__device__ __forceinline__ void pool_unit(const C& c, const PoolDev& g, int64_t f, int64_t b,
                                          float t, int normalize, float& dmax) {
  const int64_t p0 = g.ch_begin[f], p1 = g.ch_begin[f + 1];
  float old[2], vt[2];
  float sums0 = 0.0f, max1 = -INFINITY;
  for (int64_t i = p0; i < p1; ++i) {
    c.load(edge_ref(g.ch[i]), 2, b, old, vt);
    sums0 += vt[0];
    max1 = fmaxp(max1, vt[1] - vt[0]);
  }
  int64_t arg = p1 - 1;
  {
    int64_t last = -1;
    for (int64_t i = p0; i < p1; ++i) {
      c.load(edge_ref(g.ch[i]), 2, b, old, vt);
      if (vt[1] - vt[0] == max1) last = i;
    }
    if (last >= 0) arg = last;
  }
  const EdgeRef ri = edge_ref(g.ind[f]);
  float iold[2], ivt[2];
  c.load(ri, 2, b, iold, ivt);
  const float pi_one = ivt[1];
  const float pi_diff = ivt[1] - ivt[0];
  float max2 = -INFINITY, pi_mdiff, fl = 0.0f, am = 0.0f;
  if (T0) {
    for (int64_t i = p0; i < p1; ++i) {
      c.load(edge_ref(g.ch[i]), 2, b, old, vt);
      max2 = fmaxp(max2, (i == arg) ? -INFINITY : vt[1] - vt[0]);
    }
    pi_mdiff = max1;
  } else {
    float se = 0.0f;
    for (int64_t i = p0; i < p1; ++i) {
      c.load(edge_ref(g.ch[i]), 2, b, old, vt);
      se += expf(div_t((vt[1] - vt[0]) - max1, t));
    }
    pi_mdiff = t * logf(se) + max1;
    fl = logaddexp_t(pi_mdiff, -pi_diff, t);
    // -logsumexps_with_temp of the diffs with the argmax replaced by -pi_diff (pool.py:416-425)
    float mw = -INFINITY;
    for (int64_t i = p0; i < p1; ++i) {
      c.load(edge_ref(g.ch[i]), 2, b, old, vt);
      mw = fmaxp(mw, (i == arg) ? -pi_diff : vt[1] - vt[0]);
    }
    float sw = 0.0f;
    for (int64_t i = p0; i < p1; ++i) {
      c.load(edge_ref(g.ch[i]), 2, b, old, vt);
      const float w = (i == arg) ? -pi_diff : vt[1] - vt[0];
      sw += expf(div_t(w - mw, t));
    }
    am = -(t * logf(sw) + mw);
  }
  const bool single = (p1 - p0) == 1;
  for (int64_t i = p0; i < p1; ++i) {
    const EdgeRef r = edge_ref(g.ch[i]);
    c.load(r, 2, b, old, vt);
    const float dif = vt[1] - vt[0];
    float mdiff;
    if (T0) {
      mdiff = fminp(pi_diff, -(i == arg ? max2 : max1));
    } else {
      mdiff = (i == arg) ? am : -logminusexp_t(fl, dif, t, 1e-30f);
    }
    float ones = (sums0 + pi_one) - vt[0];
    if (single) {
      mdiff = pi_diff;
      ones = pi_one;
    }
    const float s1 = normalize ? mdiff : ones;
    const float s0 = normalize ? 0.0f : ones - mdiff;
    c.store(r, 2, old, [&](int s) { return s == 0 ? s0 : s1; }, b, dmax);
  }
  const float i1 = normalize ? pi_mdiff : sums0 + pi_mdiff;
  const float i0 = normalize ? 0.0f : sums0;
  c.store(ri, 2, iold, [&](int s) { return s == 0 ? i0 : i1; }, b, dmax);
}

template <bool T0, class C>
__global__ void __launch_bounds__(256) pool_kernel(C c, PoolDev g, int64_t B, float t,
                                                   int normalize, unsigned* deltas) {
  pdl_begin();
  const Lane l = lane(B);
  float dmax = 0.0f;
  if (l.valid) {
    for (int64_t f = l.u0; f < g.count; f += l.ustep) pool_unit<T0>(c, g, f, l.b, t, normalize, dmax);
  }
  block_max_to(deltas, l, dmax);
}

// ----------------------------------------------------------------------------- 4 instances per thread
// The two kernels that carry binary pairwise graphs (RBM, Ising) also come in a form where every
// thread owns 4 consecutive instances (B % 4 == 0): 128-bit loads and stores, index and address
// work shared by 4 instances, 4 independent dependency chains. Per instance the arithmetic is
// exactly the scalar kernels'.

struct Lane4 {
  int64_t b;  // first of 4 instances
  bool valid;
  int64_t u0, ustep;
};

__device__ __forceinline__ Lane4 lane4(int64_t B) {
  Lane4 l;
  l.b = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 4;
  l.valid = l.b < B;
  l.u0 = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  l.ustep = (int64_t)gridDim.y * blockDim.y;
  return l;
}

__device__ __forceinline__ void block_max4_to(unsigned* dst, const Lane4& l, float4 v) {
  __shared__ float4 red[256];
  const int tx = threadIdx.x, ty = threadIdx.y, bx = blockDim.x;
  red[ty * bx + tx] = v;
  __syncthreads();
  for (int s = blockDim.y / 2; s > 0; s >>= 1) {
    if (ty < s) {
      float4 a = red[ty * bx + tx];
      const float4 c = red[(ty + s) * bx + tx];
      a.x = fmaxp(a.x, c.x);
      a.y = fmaxp(a.y, c.y);
      a.z = fmaxp(a.z, c.z);
      a.w = fmaxp(a.w, c.w);
      red[ty * bx + tx] = a;
    }
    __syncthreads();
  }
  if (ty == 0 && l.valid && dst != nullptr) {
    const float4 a = red[tx];
    atomicMax(dst + l.b + 0, __float_as_uint(a.x));
    atomicMax(dst + l.b + 1, __float_as_uint(a.y));
    atomicMax(dst + l.b + 2, __float_as_uint(a.z));
    atomicMax(dst + l.b + 3, __float_as_uint(a.w));
  }
}

// One instance of a dense 2x2 pairwise factor with both edges binary: c1 / c2 are the compressed
// current messages to variables 1 and 2, a0 a1 / b0 b1 their variable sums, p00..p11 the table.
// Same operations, in the same order, as pairwise_body<2, 2> with Fused.
template <bool T0>
__device__ __forceinline__ void pair22(float c1, float c2, float a0, float a1, float b0, float b1,
                                       float p00, float p01, float p10, float p11, float t,
                                       float d, float omd, float& n1, float& n2, float& dmax) {
  float o10, o11, o20, o21;
  decode2(c1, o10, o11);
  decode2(c2, o20, o21);
  const float v10 = a0 - o10, v11 = a1 - o11, v20 = b0 - o20, v21 = b1 - o21;
  const float s00 = ((0.0f + v10) + v20) + p00;
  const float s01 = ((0.0f + v10) + v21) + p01;
  const float s10 = ((0.0f + v11) + v20) + p10;
  const float s11 = ((0.0f + v11) + v21) + p11;
  // max(max(-inf, a), b) == max(a, b) for every input, NaN included
  const float m10 = fmaxp(s00, s01);
  const float m11 = fmaxp(s10, s11);
  const float m20 = fmaxp(s00, s10);
  const float m21 = fmaxp(s01, s11);
  float f10, f11, f20, f21;
  if (T0) {
    f10 = m10 - v10;
    f11 = m11 - v11;
    f20 = m20 - v20;
    f21 = m21 - v21;
  } else {
    const float e10 = (0.0f + expf(div_t(s00 - m10, t))) + expf(div_t(s01 - m10, t));
    const float e11 = (0.0f + expf(div_t(s10 - m11, t))) + expf(div_t(s11 - m11, t));
    const float e20 = (0.0f + expf(div_t(s00 - m20, t))) + expf(div_t(s10 - m20, t));
    const float e21 = (0.0f + expf(div_t(s01 - m21, t))) + expf(div_t(s11 - m21, t));
    f10 = (t * logf(e10) + m10) - v10;
    f11 = (t * logf(e11) + m11) - v11;
    f20 = (t * logf(e20) + m20) - v20;
    f21 = (t * logf(e21) + m21) - v21;
  }
  {
    const float q0 = d * o10 + omd * f10, q1 = d * o11 + omd * f11;
    const float m = fmaxp(q0, q1);
    const float w0 = fmaxp(q0 - m, kMsgNegInf), w1 = fmaxp(q1 - m, kMsgNegInf);
    n1 = encode2(w0, w1);
    dmax = fmaxp(dmax, fabsf(w0 - o10));
    dmax = fmaxp(dmax, fabsf(w1 - o11));
  }
  {
    const float q0 = d * o20 + omd * f20, q1 = d * o21 + omd * f21;
    const float m = fmaxp(q0, q1);
    const float w0 = fmaxp(q0 - m, kMsgNegInf), w1 = fmaxp(q1 - m, kMsgNegInf);
    n2 = encode2(w0, w1);
    dmax = fmaxp(dmax, fabsf(w0 - o20));
    dmax = fmaxp(dmax, fabsf(w1 - o21));
  }
}

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }

// Each unit lane walks a contiguous chunk of factors, so consecutive factors that share their
// first variable (a PairwiseFactorGroup built row by row) reuse its variable sums from registers.
template <bool T0>
__global__ void __launch_bounds__(256, 4) pairwise22_x4_kernel(Fused c, PairwiseDev p, float t,
                                                            unsigned* deltas) {
  pdl_begin();
  const int64_t B = c.B;
  const Lane4 l = lane4(B);
  float4 dm = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (l.valid) {
    const int64_t b = l.b;
    const int64_t chunk = (p.count + l.ustep - 1) / l.ustep;
    const int64_t u_begin = l.u0 * chunk;
    const int64_t u_end = u_begin + chunk < p.count ? u_begin + chunk : p.count;
    int32_t za = -1;
    float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), a1 = a0;
    for (int64_t u = u_begin; u < u_end; ++u) {
      const int4 q = __ldg(p.rec + u);
      const int64_t k0 = __ldg(p.cfg_begin + u);
      const float4 c1 = ld4(c.cur + (int64_t)q.y * B + b);
      const float4 c2 = ld4(c.cur + ((int64_t)q.y + 1) * B + b);
      if (q.z != za) {
        za = q.z;
        a0 = ld4(c.vsum + (int64_t)q.z * B + b);
        a1 = ld4(c.vsum + ((int64_t)q.z + 1) * B + b);
      }
      const float4 b0 = ld4(c.vsum + (int64_t)q.w * B + b);
      const float4 b1 = ld4(c.vsum + ((int64_t)q.w + 1) * B + b);
      float4 p00, p01, p10, p11;
      if (c.lpb == 0) {
        float4 pp;
        if ((k0 & 3) == 0) {  // 16-byte aligned table: one vector load
          pp = __ldg(reinterpret_cast<const float4*>(c.lp + k0));
        } else {
          pp = make_float4(__ldg(c.lp + k0), __ldg(c.lp + k0 + 1), __ldg(c.lp + k0 + 2),
                           __ldg(c.lp + k0 + 3));
        }
        p00 = make_float4(pp.x, pp.x, pp.x, pp.x);
        p01 = make_float4(pp.y, pp.y, pp.y, pp.y);
        p10 = make_float4(pp.z, pp.z, pp.z, pp.z);
        p11 = make_float4(pp.w, pp.w, pp.w, pp.w);
      } else {
        p00 = ld4(c.lp + k0 * B + b);
        p01 = ld4(c.lp + (k0 + 1) * B + b);
        p10 = ld4(c.lp + (k0 + 2) * B + b);
        p11 = ld4(c.lp + (k0 + 3) * B + b);
      }
      float4 n1, n2;
      pair22<T0>(c1.x, c2.x, a0.x, a1.x, b0.x, b1.x, p00.x, p01.x, p10.x, p11.x, t, c.d, c.omd,
                 n1.x, n2.x, dm.x);
      pair22<T0>(c1.y, c2.y, a0.y, a1.y, b0.y, b1.y, p00.y, p01.y, p10.y, p11.y, t, c.d, c.omd,
                 n1.y, n2.y, dm.y);
      pair22<T0>(c1.z, c2.z, a0.z, a1.z, b0.z, b1.z, p00.z, p01.z, p10.z, p11.z, t, c.d, c.omd,
                 n1.z, n2.z, dm.z);
      pair22<T0>(c1.w, c2.w, a0.w, a1.w, b0.w, b1.w, p00.w, p01.w, p10.w, p11.w, t, c.d, c.omd,
                 n1.w, n2.w, dm.w);
      st4(c.nxt + (int64_t)q.y * B + b, n1);
      st4(c.nxt + ((int64_t)q.y + 1) * B + b, n2);
    }
  }
  block_max4_to(deltas, l, dm);
}

// ----------------------------------------------------------------------------- unary factors
// A generic Enum factor that is unary on a binary variable with configs (0), (1) in that order
// (Plan::unary2): the operations of enum_generic_unit for it, in the same order (s = (0 + v) + p,
// its maximum with -inf, at T > 0 exp((s - max) / T) added to 0, then Fused::store's damping,
// normalisation and clip), without its per-thread arrays. c is the compressed current message,
// a0 / a1 the variable's sums, p0 / p1 the two potentials.
template <bool T0>
__device__ __forceinline__ void unary2(float c, float a0, float a1, float p0, float p1, float t,
                                       float d, float omd, float& n, float& dmax) {
  float o0, o1;
  decode2(c, o0, o1);
  const float v0 = a0 - o0, v1 = a1 - o1;
  const float s0 = (0.0f + v0) + p0, s1 = (0.0f + v1) + p1;
  const float mx0 = fmaxp(-INFINITY, s0), mx1 = fmaxp(-INFINITY, s1);
  float f0, f1;
  if (T0) {
    f0 = mx0 - v0;
    f1 = mx1 - v1;
  } else {
    const float se0 = 0.0f + expf(div_t(s0 - mx0, t));
    const float se1 = 0.0f + expf(div_t(s1 - mx1, t));
    f0 = (t * logf(se0) + mx0) - v0;
    f1 = (t * logf(se1) + mx1) - v1;
  }
  const float q0 = d * o0 + omd * f0, q1 = d * o1 + omd * f1;
  const float m = fmaxp(q0, q1);
  const float w0 = fmaxp(q0 - m, kMsgNegInf), w1 = fmaxp(q1 - m, kMsgNegInf);
  n = encode2(w0, w1);
  dmax = fmaxp(dmax, fabsf(w0 - o0));
  dmax = fmaxp(dmax, fabsf(w1 - o1));
}

struct Unary2Dev {
  const int4* __restrict__ rec;  // (first edge state, slot, first variable state, potential)
  int64_t count;
};

// 4 instances per thread (B % 4 == 0).
template <bool T0>
__global__ void __launch_bounds__(256) unary2_x4_kernel(Fused c, Unary2Dev g, float t,
                                                        unsigned* deltas) {
  pdl_begin();
  const int64_t B = c.B;
  const Lane4 l = lane4(B);
  float4 dm = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (l.valid) {
    const int64_t b = l.b;
    for (int64_t u = l.u0; u < g.count; u += l.ustep) {
      const int4 q = __ldg(g.rec + u);
      const float4 c4 = ld4(c.cur + (int64_t)q.y * B + b);
      const float4 a0 = ld4(c.vsum + (int64_t)q.z * B + b);
      const float4 a1 = ld4(c.vsum + ((int64_t)q.z + 1) * B + b);
      float4 p0, p1;
      if (c.lpb == 0) {
        const float x0 = __ldg(c.lp + (int64_t)q.w * c.lps), x1 = __ldg(c.lp + ((int64_t)q.w + 1) * c.lps);
        p0 = make_float4(x0, x0, x0, x0);
        p1 = make_float4(x1, x1, x1, x1);
      } else {
        p0 = ld4(c.lp + (int64_t)q.w * c.lps + b);
        p1 = ld4(c.lp + ((int64_t)q.w + 1) * c.lps + b);
      }
      float4 n;
      unary2<T0>(c4.x, a0.x, a1.x, p0.x, p1.x, t, c.d, c.omd, n.x, dm.x);
      unary2<T0>(c4.y, a0.y, a1.y, p0.y, p1.y, t, c.d, c.omd, n.y, dm.y);
      unary2<T0>(c4.z, a0.z, a1.z, p0.z, p1.z, t, c.d, c.omd, n.z, dm.z);
      unary2<T0>(c4.w, a0.w, a1.w, p0.w, p1.w, t, c.d, c.omd, n.w, dm.w);
      st4(c.nxt + (int64_t)q.y * B + b, n);
    }
  }
  block_max4_to(deltas, l, dm);
}

// One instance per thread.
template <bool T0>
__global__ void __launch_bounds__(256) unary2_kernel(Fused c, Unary2Dev g, float t,
                                                     unsigned* deltas) {
  pdl_begin();
  const int64_t B = c.B;
  const Lane l = lane(B);
  float dm = 0.0f;
  if (l.valid) {
    const int64_t b = l.b;
    for (int64_t u = l.u0; u < g.count; u += l.ustep) {
      const int4 q = __ldg(g.rec + u);
      float n;
      unary2<T0>(c.cur[(int64_t)q.y * B + b], c.vsum[(int64_t)q.z * B + b],
                 c.vsum[((int64_t)q.z + 1) * B + b], c.pot(q.w, b), c.pot((int64_t)q.w + 1, b),
                 t, c.d, c.omd, n, dm);
      c.nxt[(int64_t)q.y * B + b] = n;
    }
  }
  block_max_to(deltas, l, dm);
}

// ----------------------------------------------------------------------------- variable sums
// var_sums = evidence.at[var_states_for_edge_states].add(msgs) (bp.py:217): serial per variable
// state over its edge states in increasing order. Binary variables read one compressed slot per
// edge and accumulate both states. `for_each_slot` walks a unit's slots in order, either from
// affine runs (no index loads) or from the explicit list, eight loads in flight.
struct VarsumDev {
  const int32_t* __restrict__ vs;
  const int32_t* __restrict__ off;
  const int32_t* __restrict__ slots;
  const int32_t* __restrict__ run_off;
  const int4* __restrict__ runs;
  int64_t count;
};

template <int UNROLL, class Load, class Add>
__device__ __forceinline__ void for_each_slot(const VarsumDev& v, bool use_runs, int64_t u,
                                              Load load, Add add) {
  using T = decltype(load((int64_t)0));
  if (use_runs) {
    for (int32_t r = v.run_off[u]; r < v.run_off[u + 1]; ++r) {
      const int4 run = __ldg(v.runs + r);
      const int64_t first = run.x, stride = run.y;
      const int32_t len = run.z;
      int32_t k = 0;
      if (len >= 2 * UNROLL) {
        // software pipeline: the loads of the next UNROLL slots are issued before the current
        // UNROLL are added, so 2 * UNROLL loads are in flight per thread
        T cur[UNROLL], nxt[UNROLL];
#pragma unroll
        for (int q = 0; q < UNROLL; ++q) cur[q] = load(first + (int64_t)q * stride);
        k = UNROLL;
        for (; k + UNROLL <= len; k += UNROLL) {
#pragma unroll
          for (int q = 0; q < UNROLL; ++q) nxt[q] = load(first + (int64_t)(k + q) * stride);
#pragma unroll
          for (int q = 0; q < UNROLL; ++q) add(cur[q]);
#pragma unroll
          for (int q = 0; q < UNROLL; ++q) cur[q] = nxt[q];
        }
#pragma unroll
        for (int q = 0; q < UNROLL; ++q) add(cur[q]);
      }
      for (; k + UNROLL <= len; k += UNROLL) {
        T c[UNROLL];
#pragma unroll
        for (int q = 0; q < UNROLL; ++q) c[q] = load(first + (int64_t)(k + q) * stride);
#pragma unroll
        for (int q = 0; q < UNROLL; ++q) add(c[q]);
      }
      for (; k < len; ++k) add(load(first + (int64_t)k * stride));
    }
  } else {
    const int32_t k1 = v.off[u + 1];
    int32_t k = v.off[u];
    for (; k + UNROLL <= k1; k += UNROLL) {
      T c[UNROLL];
#pragma unroll
      for (int q = 0; q < UNROLL; ++q) c[q] = load((int64_t)__ldg(v.slots + k + q));
#pragma unroll
      for (int q = 0; q < UNROLL; ++q) add(c[q]);
    }
    for (; k < k1; ++k) add(load((int64_t)__ldg(v.slots + k)));
  }
}

// Variable sums of unit u (binary: both states), instance b.
__device__ __forceinline__ void varsum_binary_unit(const VarsumDev& v, bool use_runs, int64_t u,
                                                   int64_t b, const float* __restrict__ msgs,
                                                   const float* __restrict__ ev, int64_t evs,
                                                   int64_t evb, float* __restrict__ vsum,
                                                   int64_t B) {
  const float* col = msgs + b;
  const int64_t v0 = v.vs[u];
  float s0 = ev[v0 * evs + b * evb];
  float s1 = ev[(v0 + 1) * evs + b * evb];
  for_each_slot<16>(v, use_runs, u, [&](int64_t slot) { return col[slot * B]; },
                    [&](float c) {
                      float m0, m1;
                      decode2(c, m0, m1);
                      s0 += m0;
                      s1 += m1;
                    });
  vsum[v0 * B + b] = s0;
  vsum[(v0 + 1) * B + b] = s1;
}

__device__ __forceinline__ void varsum_other_unit(const VarsumDev& v, bool use_runs, int64_t u,
                                                  int64_t b, const float* __restrict__ msgs,
                                                  const float* __restrict__ ev, int64_t evs,
                                                  int64_t evb, float* __restrict__ vsum, int64_t B) {
  const float* col = msgs + b;
  const int64_t vv = v.vs[u];
  float s = ev[vv * evs + b * evb];
  for_each_slot<8>(v, use_runs, u, [&](int64_t slot) { return col[slot * B]; },
                   [&](float c) { s += c; });
  vsum[vv * B + b] = s;
}

// At least three blocks per SM, i.e. up to 85 registers: the compiler then keeps the 16-slot
// load batches of both buffers in flight (72 registers), which beat four blocks per SM at 64
// registers on the RBM's 784- and 500-slot chains (about 1 ms per 200-iteration step).
__global__ void __launch_bounds__(256, 3) varsum_binary_kernel(VarsumDev v, bool use_runs,
                                                            const float* __restrict__ msgs,
                                                            const float* __restrict__ ev,
                                                            int64_t evs, int64_t evb,
                                                            float* __restrict__ vsum, int64_t B) {
  pdl_begin();
  const Lane l = lane(B);
  if (!l.valid) return;
  for (int64_t u = l.u0; u < v.count; u += l.ustep)
    varsum_binary_unit(v, use_runs, u, l.b, msgs, ev, evs, evb, vsum, B);
}

__global__ void __launch_bounds__(256) varsum_other_kernel(VarsumDev v, bool use_runs,
                                                           const float* __restrict__ msgs,
                                                           const float* __restrict__ ev,
                                                           int64_t evs, int64_t evb,
                                                           float* __restrict__ vsum, int64_t B) {
  pdl_begin();
  const Lane l = lane(B);
  if (!l.valid) return;
  for (int64_t u = l.u0; u < v.count; u += l.ustep)
    varsum_other_unit(v, use_runs, u, l.b, msgs, ev, evs, evb, vsum, B);
}

// Variable sums of non-binary variables by variable (VarsumSet::byvar_*): per (variable state,
// instance) evidence plus the messages of the variable's edges in edge order, with the state's
// slot at the edge's first slot + state: no per-state index. Consecutive units are consecutive
// states of one variable, whose slots are consecutive.
__global__ void __launch_bounds__(256) varsum_byvar_kernel(
    const int4* __restrict__ grp, int n_groups, int64_t units, const int32_t* __restrict__ vs0,
    const int32_t* __restrict__ eoff, const int32_t* __restrict__ eslot,
    const float* __restrict__ msgs, const float* __restrict__ ev, int64_t evs, int64_t evb,
    float* __restrict__ vsum, int64_t B) {
  pdl_begin();
  const Lane l = lane(B);
  if (!l.valid) return;
  const int64_t b = l.b;
  int g = 0;
  for (int64_t u = l.u0; u < units; u += l.ustep) {
    while (g + 1 < n_groups && u >= grp[g + 1].y) ++g;
    const int4 gr = grp[g];
    const int32_t local = (int32_t)(u - gr.y);
    const int32_t var = gr.z + local / gr.x, st = local % gr.x;
    const int64_t v = (int64_t)vs0[var] + st;
    float sum = evb == 0 ? ev[v * evs] : ev[v * evs + b];
    const int32_t k1 = eoff[var + 1];
    for (int32_t k = eoff[var]; k < k1; ++k) sum += msgs[((int64_t)eslot[k] + st) * B + b];
    vsum[v * B + b] = sum;
  }
}

// Binary variable sums, 4 instances per thread, sixteen slots in flight.
__global__ void __launch_bounds__(256) varsum_binary_x4_kernel(VarsumDev v, bool use_runs,
                                                               const float* __restrict__ msgs,
                                                               const float* __restrict__ ev,
                                                               int64_t evs, int64_t evb,
                                                               float* __restrict__ vsum, int64_t B) {
  pdl_begin();
  const Lane4 l = lane4(B);
  if (!l.valid) return;
  const int64_t b = l.b;
  const float* col = msgs + b;
  for (int64_t u = l.u0; u < v.count; u += l.ustep) {
    const int64_t v0 = v.vs[u];
    float4 s0, s1;
    if (evb == 0) {
      const float e0 = ev[v0 * evs], e1 = ev[(v0 + 1) * evs];
      s0 = make_float4(e0, e0, e0, e0);
      s1 = make_float4(e1, e1, e1, e1);
    } else {
      s0 = ld4(ev + v0 * evs + b);
      s1 = ld4(ev + (v0 + 1) * evs + b);
    }
    for_each_slot<16>(v, use_runs, u, [&](int64_t slot) { return ld4(col + slot * B); },
                      [&](float4 c4) {
                        float m0, m1;
                        decode2(c4.x, m0, m1);
                        s0.x += m0;
                        s1.x += m1;
                        decode2(c4.y, m0, m1);
                        s0.y += m0;
                        s1.y += m1;
                        decode2(c4.z, m0, m1);
                        s0.z += m0;
                        s1.z += m1;
                        decode2(c4.w, m0, m1);
                        s0.w += m0;
                        s1.w += m1;
                      });
    st4(vsum + v0 * B + b, s0);
    st4(vsum + (v0 + 1) * B + b, s1);
  }
}

// Binary variable sums, 2 instances per thread (float2), sixteen slots in flight: half the
// threads of the one-instance kernel, so a batch like the RBM's (1,284 variables x 128 instances)
// fits in one wave of resident blocks instead of leaving its longest chains to a second one.
__global__ void __launch_bounds__(256, 3) varsum_binary_x2_kernel(VarsumDev v, bool use_runs,
                                                                  const float* __restrict__ msgs,
                                                                  const float* __restrict__ ev,
                                                                  int64_t evs, int64_t evb,
                                                                  float* __restrict__ vsum,
                                                                  int64_t B) {
  pdl_begin();
  const int64_t b = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 2;
  if (b >= B) return;
  const int64_t u0 = (int64_t)blockIdx.y * blockDim.y + threadIdx.y;
  const int64_t ustep = (int64_t)gridDim.y * blockDim.y;
  const float* col = msgs + b;
  for (int64_t u = u0; u < v.count; u += ustep) {
    const int64_t v0 = v.vs[u];
    float2 s0, s1;
    if (evb == 0) {
      const float e0 = ev[v0 * evs], e1 = ev[(v0 + 1) * evs];
      s0 = make_float2(e0, e0);
      s1 = make_float2(e1, e1);
    } else {
      s0 = *reinterpret_cast<const float2*>(ev + v0 * evs + b);
      s1 = *reinterpret_cast<const float2*>(ev + (v0 + 1) * evs + b);
    }
    for_each_slot<16>(v, use_runs, u,
                      [&](int64_t slot) { return *reinterpret_cast<const float2*>(col + slot * B); },
                      [&](float2 c2) {
                        float m0, m1;
                        decode2(c2.x, m0, m1);
                        s0.x += m0;
                        s1.x += m1;
                        decode2(c2.y, m0, m1);
                        s0.y += m0;
                        s1.y += m1;
                      });
    *reinterpret_cast<float2*>(vsum + v0 * B + b) = s0;
    *reinterpret_cast<float2*>(vsum + (v0 + 1) * B + b) = s1;
  }
}

// ----------------------------------------------------------------------------- small graphs
// Graphs whose messages, variable sums and evidence fit in shared memory (Ising 50x50: 10,000
// slots) run every iteration in one launch: one CTA per instance keeps its state on chip and
// separates the variable-sum and factor phases with __syncthreads, so an iteration costs two
// block barriers instead of two kernel launches. The per-factor work is the same device code as
// the multi-kernel path (Fused context over shared memory, one instance per CTA).
constexpr int kSmallMaxBuckets = 4;
constexpr int kSmallThreads = 1024;

// Fused with each variable's two sums formed inline, for graphs whose edges are all binary: the
// evidence plus the variable's compressed slots in the order of varsum_binary_unit (the same
// float additions, so the same values as a variable-sum pass), so an iteration needs no phase
// (and no barrier) between the variable sums and the factor updates.
struct FusedInline : Fused {
  VarsumDev vb;
  bool runs;
  const int32_t* __restrict__ unit_of_vs;
  const float* __restrict__ ev;
  int64_t evs, evb;

  __device__ __forceinline__ void load(const EdgeRef& r, int k, int64_t b, float* old,
                                       float* vt) const {
    (void)k;  // every edge of an eligible graph is binary
    decode2(cur[r.slot * B + b], old[0], old[1]);
    const int64_t u = __ldg(unit_of_vs + r.vs0);
    float s0 = ev[r.vs0 * evs + b * evb];
    float s1 = ev[(r.vs0 + 1) * evs + b * evb];
    const float* col = cur + b;
    for_each_slot<16>(vb, runs, u, [&](int64_t slot) { return col[slot * B]; },
                      [&](float c) {
                        float m0, m1;
                        decode2(c, m0, m1);
                        s0 += m0;
                        s1 += m1;
                      });
    vt[0] = s0 - old[0];
    vt[1] = s1 - old[1];
  }
};

struct SmallGraph {
  const int32_t* unit_of_vs;  // inline variable sums (Plan::vb_unit_of_vs), or null
  PairwiseDev pw[kSmallMaxBuckets];
  int n_pw;
  EnumGenericDev eg;
  LogicalDev lg[2];
  PoolDev pool;
  VarsumDev vb, vo;
  bool vb_runs, vo_runs;
  int64_t num_slots, num_var_states;
  const float* ev;  // run layout: [N_vs][B] (evb = 1, evs = B) or shared [N_vs]
  int64_t evs, evb;
  const float* lp;
  int64_t lps, lpb;
  float d, omd;
};

__device__ __forceinline__ float block_max_all(float v, float* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxp(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
  if (ln == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = ln < (int)(blockDim.x >> 5) ? red[ln] : 0.0f;
    for (int o = 16; o > 0; o >>= 1) v = fmaxp(v, __shfl_xor_sync(0xffffffffu, v, o));
  }
  return v;  // valid in thread 0
}

template <bool T0, int MAXES>
__global__ void __launch_bounds__(kSmallThreads) small_graph_kernel(SmallGraph g, int64_t B,
                                                                    int64_t iters, float t,
                                                                    bool low_t,
                                                                    float* __restrict__ msgs,
                                                                    unsigned* __restrict__ dacc) {
  extern __shared__ float sm[];
  __shared__ float red[32];
  const int64_t inst = blockIdx.x;
  const int tid = threadIdx.x, nt = blockDim.x;
  float* cur = sm;
  float* nxt = sm + g.num_slots;
  float* vsum = nxt + g.num_slots;
  float* evs = vsum + g.num_var_states;
  for (int64_t i = tid; i < g.num_slots; i += nt) cur[i] = msgs[i * B + inst];
  for (int64_t i = tid; i < g.num_var_states; i += nt) evs[i] = g.ev[i * g.evs + inst * g.evb];
  __syncthreads();
  Fused c;
  c.vsum = vsum;
  c.lp = g.lp + inst * g.lpb;
  c.lps = g.lps;
  c.lpb = 0;
  c.B = 1;
  c.d = g.d;
  c.omd = g.omd;
  for (int64_t it = 0; it < iters; ++it) {
    for (int64_t u = tid; u < g.vb.count; u += nt)
      varsum_binary_unit(g.vb, g.vb_runs, u, 0, cur, evs, 1, 0, vsum, 1);
    for (int64_t u = tid; u < g.vo.count; u += nt)
      varsum_other_unit(g.vo, g.vo_runs, u, 0, cur, evs, 1, 0, vsum, 1);
    __syncthreads();
    c.cur = cur;
    c.nxt = nxt;
    float dmax = 0.0f;
    for (int q = 0; q < g.n_pw; ++q) {
      const PairwiseDev& p = g.pw[q];
      for (int64_t u = tid; u < p.count; u += nt) {
        EdgeRef r1, r2;
        pairwise_refs(p, __ldg(p.rec + u), r1, r2);
        const int64_t k0 = __ldg(p.cfg_begin + u);
        if (p.n1 == 2 && p.n2 == 2) {
          pairwise_body<2, 2, T0>(c, r1, r2, k0, 2, 2, 0, t, dmax);
        } else {
          pairwise_body<0, 0, T0>(c, r1, r2, k0, p.n1, p.n2, 0, t, dmax);
        }
      }
    }
    for (int64_t f = tid; f < g.eg.count; f += nt) enum_generic_unit<MAXES, T0>(c, g.eg, f, 0, t, dmax);
    for (int w = 0; w < 2; ++w)
      for (int64_t f = tid; f < g.lg[w].count; f += nt)
        logical_unit<T0>(c, g.lg[w], f, 0, t, low_t, 1, dmax);
    for (int64_t f = tid; f < g.pool.count; f += nt) pool_unit<T0>(c, g.pool, f, 0, t, 1, dmax);
    const float m = block_max_all(dmax, red);
    if (tid == 0) dacc[it * B + inst] = __float_as_uint(m);
    __syncthreads();
    float* sw = cur;
    cur = nxt;
    nxt = sw;
  }
  for (int64_t i = tid; i < g.num_slots; i += nt) msgs[i * B + inst] = cur[i];
}

// ----------------------------------------------------------------------------- clustered graphs
// One thread-block cluster per instance: the cluster's CTAs split the variable-sum and factor
// phases between them and meet at hardware cluster barriers (barrier.cluster with release /
// acquire semantics, which order their global-memory writes), so an iteration costs two cluster
// barriers and the work of one instance is spread over up to 16 SMs. State stays in the run
// layout in global memory (L2-resident for the graphs this path is chosen for).
// INL: the variable sums are formed inline by the factor units (FusedInline; all-binary Enum
// graphs of low degree), which leaves one cluster barrier per iteration.
template <bool T0, int MAXES, bool INL>
__global__ void __launch_bounds__(kSmallThreads) cluster_graph_kernel(SmallGraph g, int64_t B,
                                                                      int64_t iters, float t,
                                                                      bool low_t, float* m0,
                                                                      float* m1, float* vsum,
                                                                      unsigned* __restrict__ dacc) {
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  __shared__ float red[32];
  const int64_t csize = (int64_t)cluster.num_blocks();
  const int64_t inst = blockIdx.x / csize;
  const int64_t tid = (int64_t)cluster.block_rank() * blockDim.x + threadIdx.x;
  const int64_t nt = csize * blockDim.x;
  typename std::conditional<INL, FusedInline, Fused>::type c;
  c.vsum = vsum;
  c.lp = g.lp;
  c.lps = g.lps;
  c.lpb = g.lpb;
  c.B = B;
  c.d = g.d;
  c.omd = g.omd;
  if constexpr (INL) {
    c.vb = g.vb;
    c.runs = g.vb_runs;
    c.unit_of_vs = g.unit_of_vs;
    c.ev = g.ev;
    c.evs = g.evs;
    c.evb = g.evb;
  }
  float* cur = m0;
  float* nxt = m1;
  for (int64_t it = 0; it < iters; ++it) {
    if constexpr (!INL) {
      for (int64_t u = tid; u < g.vb.count; u += nt)
        varsum_binary_unit(g.vb, g.vb_runs, u, inst, cur, g.ev, g.evs, g.evb, vsum, B);
      for (int64_t u = tid; u < g.vo.count; u += nt)
        varsum_other_unit(g.vo, g.vo_runs, u, inst, cur, g.ev, g.evs, g.evb, vsum, B);
      cluster.sync();
    }
    c.cur = cur;
    c.nxt = nxt;
    float dmax = 0.0f;
    for (int q = 0; q < g.n_pw; ++q) {
      const PairwiseDev& p = g.pw[q];
      for (int64_t u = tid; u < p.count; u += nt) {
        EdgeRef r1, r2;
        pairwise_refs(p, __ldg(p.rec + u), r1, r2);
        const int64_t k0 = __ldg(p.cfg_begin + u);
        if (p.n1 == 2 && p.n2 == 2) {
          pairwise_body<2, 2, T0>(c, r1, r2, k0, 2, 2, inst, t, dmax);
        } else {
          pairwise_body<0, 0, T0>(c, r1, r2, k0, p.n1, p.n2, inst, t, dmax);
        }
      }
    }
    for (int64_t f = tid; f < g.eg.count; f += nt)
      enum_generic_unit<MAXES, T0>(c, g.eg, f, inst, t, dmax);
    for (int w = 0; w < 2; ++w)
      for (int64_t f = tid; f < g.lg[w].count; f += nt)
        logical_unit<T0>(c, g.lg[w], f, inst, t, low_t, 1, dmax);
    for (int64_t f = tid; f < g.pool.count; f += nt) pool_unit<T0>(c, g.pool, f, inst, t, 1, dmax);
    const float m = block_max_all(dmax, red);
    if (threadIdx.x == 0) atomicMax(dacc + it * B + inst, __float_as_uint(m));
    cluster.sync();
    float* sw = cur;
    cur = nxt;
    nxt = sw;
  }
}

// Flat beliefs from caller-layout arrays ([B, n] rows): inferer.py:218-222.
__global__ void __launch_bounds__(256) beliefs_kernel(const int32_t* __restrict__ vs_off,
                                                      const int32_t* __restrict__ vs_edges,
                                                      int64_t nvs, const float* __restrict__ msgs,
                                                      int64_t ms, const float* __restrict__ ev,
                                                      int64_t evs, float* __restrict__ out,
                                                      int64_t B) {
  const Lane l = lane(B);
  if (!l.valid) return;
  const int64_t b = l.b;
  for (int64_t u = l.u0; u < nvs; u += l.ustep) {
    float s = ev[b * evs + u];
    for (int32_t k = vs_off[u]; k < vs_off[u + 1]; ++k) s += msgs[b * ms + vs_edges[k]];
    out[b * nvs + u] = s;
  }
}

// ----------------------------------------------------------------------------- layout / misc
// normalize_and_clip_msgs (bp.py:222-260) of the caller's initial messages (already transposed to
// edge-state-major, `src`), packed into slots (`dst`), one (edge, instance) per thread.
__global__ void __launch_bounds__(256) normalize_pack_kernel(const int32_t* __restrict__ edge_start,
                                                             const int32_t* __restrict__ edge_slot,
                                                             int64_t ne,
                                                             const float* __restrict__ src,
                                                             float* __restrict__ dst, int64_t B) {
  const Lane l = lane(B);
  if (!l.valid) return;
  const int64_t b = l.b;
  for (int64_t u = l.u0; u < ne; u += l.ustep) {
    const int64_t s0 = edge_start[u], k = edge_start[u + 1] - s0, slot = edge_slot[u];
    float m = -INFINITY;
    for (int64_t i = 0; i < k; ++i) m = fmaxp(m, src[(s0 + i) * B + b]);
    if (k == 2) {
      const float v0 = fmaxp(src[s0 * B + b] - m, kMsgNegInf);
      const float v1 = fmaxp(src[(s0 + 1) * B + b] - m, kMsgNegInf);
      dst[slot * B + b] = encode2(v0, v1);
    } else {
      for (int64_t i = 0; i < k; ++i)
        dst[(slot + i) * B + b] = fmaxp(src[(s0 + i) * B + b] - m, kMsgNegInf);
    }
  }
}

// slots -> edge-state-major messages.
__global__ void __launch_bounds__(256) unpack_kernel(const int32_t* __restrict__ edge_start,
                                                     const int32_t* __restrict__ edge_slot,
                                                     int64_t ne, const float* __restrict__ src,
                                                     float* __restrict__ dst, int64_t B) {
  const Lane l = lane(B);
  if (!l.valid) return;
  const int64_t b = l.b;
  for (int64_t u = l.u0; u < ne; u += l.ustep) {
    const int64_t s0 = edge_start[u], k = edge_start[u + 1] - s0, slot = edge_slot[u];
    if (k == 2) {
      float m0, m1;
      decode2(src[slot * B + b], m0, m1);
      dst[s0 * B + b] = m0;
      dst[(s0 + 1) * B + b] = m1;
    } else {
      for (int64_t i = 0; i < k; ++i) dst[(s0 + i) * B + b] = src[(slot + i) * B + b];
    }
  }
}

__device__ __forceinline__ float clip_lp(float x) { return fminp(fmaxp(x, -kLpMaxAbs), kLpMaxAbs); }

// dst[i * B + b] = src[b * sstride + i] for i < n, b < B (optionally clipped), via 32x32 tiles.
__global__ void to_inner_kernel(const float* __restrict__ src, int64_t sstride, int64_t n,
                                int64_t B, float* __restrict__ dst, int clip) {
  __shared__ float tile[32][33];
  const int64_t i0 = (int64_t)blockIdx.x * 32, b0 = (int64_t)blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t b = b0 + r, i = i0 + threadIdx.x;
    if (b < B && i < n) {
      const float v = src[b * sstride + i];
      tile[r][threadIdx.x] = clip ? clip_lp(v) : v;
    }
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t i = i0 + r, b = b0 + threadIdx.x;
    if (b < B && i < n) dst[i * B + b] = tile[threadIdx.x][r];
  }
}

// Perturbed evidence of pgbp_run_perturbed: v = base + scale * G[b * n + i], G the Gumbel stream
// of `key` (pgbp_gumbel.h) and base = src[b * sstride + i] (0 when src is null), written to
// dst[i * B + b] (the run layout) and, when out is not null, to out[b * n + i] (the caller's),
// via 32x32 tiles. Every draw is computed once.
__global__ void to_inner_gumbel_kernel(const float* __restrict__ src, int64_t sstride, int64_t n,
                                       int64_t B, uint64_t key, float scale,
                                       float* __restrict__ dst, float* __restrict__ out) {
  __shared__ float tile[32][33];
  const int64_t i0 = (int64_t)blockIdx.x * 32, b0 = (int64_t)blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t b = b0 + r, i = i0 + threadIdx.x;
    if (b < B && i < n) {
      const float base = src != nullptr ? src[b * sstride + i] : 0.0f;
      const float v = base + scale * gumbel_draw(key, (uint64_t)(b * n + i));
      tile[r][threadIdx.x] = v;
      if (out != nullptr) out[b * n + i] = v;
    }
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t i = i0 + r, b = b0 + threadIdx.x;
    if (b < B && i < n) dst[i * B + b] = tile[threadIdx.x][r];
  }
}

// out[c] = G[c0 + c], c < count: the Gumbel stream of `key` (pgbp_gumbel).
__global__ void gumbel_fill_kernel(uint64_t key, int64_t c0, int64_t count,
                                   float* __restrict__ out) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < count;
       c += (int64_t)gridDim.x * blockDim.x)
    out[c] = gumbel_draw(key, (uint64_t)(c0 + c));
}

// dst[b * dstride + i] = src[i * B + b]
__global__ void to_outer_kernel(const float* __restrict__ src, int64_t n, int64_t B,
                                float* __restrict__ dst, int64_t dstride) {
  __shared__ float tile[32][33];
  const int64_t i0 = (int64_t)blockIdx.x * 32, b0 = (int64_t)blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t i = i0 + r, b = b0 + threadIdx.x;
    if (b < B && i < n) tile[r][threadIdx.x] = src[i * B + b];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t b = b0 + r, i = i0 + threadIdx.x;
    if (b < B && i < n) dst[b * dstride + i] = tile[threadIdx.x][r];
  }
}

__global__ void copy_clip_kernel(const float* __restrict__ src, int64_t n, float* __restrict__ dst,
                                 int clip) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float v = src[i];
    dst[i] = clip ? clip_lp(v) : v;
  }
}

__global__ void deltas_out_kernel(const unsigned* __restrict__ acc, int64_t iters, int64_t B,
                                  float* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < iters * B;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t it = i / B, b = i % B;
    out[b * iters + it] = __uint_as_float(acc[i]);
  }
}

// States s0 .. s1 - 1 of variable v: from the plan's var_off, or, for dense [rows, k] arrays
// (var_off null), the k states of row v.
__device__ __forceinline__ void var_states(const int32_t* __restrict__ var_off, int64_t k,
                                           int64_t v, int64_t& s0, int64_t& s1) {
  if (var_off != nullptr) {
    s0 = var_off[v];
    s1 = var_off[v + 1];
  } else {
    s0 = v * k;
    s1 = s0 + k;
  }
}

// decode_map_states (inferer.py:251-264): jnp.argmax, first maximum (or first NaN) wins.
__global__ void decode_kernel(const int32_t* __restrict__ var_off, int64_t k, int64_t nv,
                              const float* __restrict__ bel, int64_t bs, int32_t* __restrict__ map,
                              int64_t B) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv * B;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / nv, v = i % nv;
    int64_t s0, s1;
    var_states(var_off, k, v, s0, s1);
    float best = s1 > s0 ? bel[b * bs + s0] : 0.0f;
    int32_t arg = 0;
    for (int64_t s = s0 + 1; s < s1; ++s) {
      const float x = bel[b * bs + s];
      if (best != best) break;
      if (x > best || x != x) {
        best = x;
        arg = (int32_t)(s - s0);
      }
    }
    map[b * nv + v] = arg;
  }
}

// get_marginals (bp.py:263-288): exp(x - logsumexp(x)) per variable, the maximum taken as 0 when
// it is not finite (so a variable whose states are all -inf gets nan, as in the reference).
__global__ void marginals_kernel(const int32_t* __restrict__ var_off, int64_t k, int64_t nv,
                                 const float* __restrict__ bel, int64_t bs, float* __restrict__ out,
                                 int64_t B, int64_t nvs) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv * B;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / nv, v = i % nv;
    int64_t s0, s1;
    var_states(var_off, k, v, s0, s1);
    float m = -INFINITY;
    for (int64_t s = s0; s < s1; ++s) m = fmaxp(m, bel[b * bs + s]);
    const float shift = isfinite(m) ? m : 0.0f;
    float se = 0.0f;
    for (int64_t s = s0; s < s1; ++s) se += expf(bel[b * bs + s] - shift);
    const float lse = logf(se) + shift;
    for (int64_t s = s0; s < s1; ++s) out[b * nvs + s] = expf(bel[b * bs + s] - lse);
  }
}

// ----------------------------------------------------------------------------- host helpers
struct Launch2 {
  dim3 grid, block;
};

Launch2 launch2(int64_t units, int64_t B, int sm_count) {
  int bx = 1;
  while (bx < B && bx < 32) bx <<= 1;
  const int by = 256 / bx;
  const int64_t gx = (B + bx - 1) / bx;
  int64_t want = (units + by - 1) / by;
  if (want < 1) want = 1;
  int64_t cap = std::max<int64_t>(1, (int64_t)sm_count * 8 / gx);
  int64_t gy = std::min<int64_t>(std::min<int64_t>(want, cap), 65535);
  Launch2 l;
  l.grid = dim3((unsigned)gx, (unsigned)gy, 1);
  l.block = dim3((unsigned)bx, (unsigned)by, 1);
  return l;
}

dim3 flat_grid(int64_t n, int sm_count) {
  int64_t g = (n + 255) / 256;
  g = std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)sm_count * 16));
  return dim3((unsigned)g);
}

void to_inner(cudaStream_t s, const float* src, int64_t sstride, int64_t n, int64_t B, float* dst,
              bool clip, int sm) {
  if (n <= 0 || B <= 0) return;
  ProfileScope ps(kProfLayout, s);
  if (B == 1) {
    copy_clip_kernel<<<flat_grid(n, sm), 256, 0, s>>>(src, n, dst, clip ? 1 : 0);
    return;
  }
  dim3 grid((unsigned)((n + 31) / 32), (unsigned)((B + 31) / 32));
  to_inner_kernel<<<grid, dim3(32, 8), 0, s>>>(src, sstride, n, B, dst, clip ? 1 : 0);
}

void to_outer(cudaStream_t s, const float* src, int64_t n, int64_t B, float* dst, int64_t dstride,
              int sm) {
  if (n <= 0 || B <= 0) return;
  ProfileScope ps(kProfLayout, s);
  if (B == 1) {
    copy_clip_kernel<<<flat_grid(n, sm), 256, 0, s>>>(src, n, dst, 0);
    return;
  }
  dim3 grid((unsigned)((n + 31) / 32), (unsigned)((B + 31) / 32));
  to_outer_kernel<<<grid, dim3(32, 8), 0, s>>>(src, n, B, dst, dstride);
}

PairwiseDev dev(const PairwiseBucket& q) {
  return PairwiseDev{q.rec, q.cfg_begin, q.count, q.n1, q.n2};
}
EnumGenericDev dev(const EnumGeneric& g) {
  return EnumGenericDev{g.es_begin,  g.n_es,    g.edge_off, g.edge_size, g.edge_slot,
                        g.edge_vs,   g.row_begin, g.n_cfg,  g.n_vars,    g.cfg_begin,
                        g.row_les,   g.count,   g.inv_begin, g.inv_off,  g.inv_cfg};
}
LogicalDev dev(const LogicalSet& g) {
  return LogicalDev{g.par_begin, g.par, g.child, g.count, g.off};
}
PoolDev dev(const PoolSet& g) { return PoolDev{g.ch_begin, g.ch, g.ind, g.count}; }

// x4 launch: lanes over groups of 4 instances.
Launch2 launch2_x4(int64_t units, int64_t B, int sm_count) { return launch2(units, B / 4, sm_count); }

template <bool T0, class C>
void launch_pairwise(cudaStream_t s, const Plan& p, const PairwiseBucket& q, const C& c, int64_t B,
                     float t, unsigned* deltas) {
  if (q.count == 0) return;
  ProfileScope ps(kProfPairwise, s);
  const Launch2 l = launch2(q.count, B, p.sm_count);
  const PairwiseDev d = dev(q);
  if (q.n1 == 2 && q.n2 == 2) {
    launch_pdl(s, l.grid, l.block, pairwise_kernel<2, 2, T0, C>, c, d, B, t, deltas);
  } else if (q.n1 == 4 && q.n2 == 4) {
    launch_pdl(s, l.grid, l.block, pairwise_kernel<4, 4, T0, C>, c, d, B, t, deltas);
  } else if (q.n1 == 8 && q.n2 == 8) {
    launch_pdl(s, l.grid, l.block, pairwise_kernel<8, 8, T0, C>, c, d, B, t, deltas);
  } else {
    launch_pdl(s, l.grid, l.block, pairwise_kernel<0, 0, T0, C>, c, d, B, t, deltas);
  }
}

// Shape of the staged kernel for a set: instances per CTA (a power of two up to 32) and configs
// per tile, within 48 KB of shared memory (four CTAs per SM).
StagedShape staged_shape(const EnumGeneric& g, int64_t B, bool t0) {
  const size_t budget = 48 * 1024;
  int ib = 1;
  while (ib * 2 <= std::min<int64_t>(B, 32)) ib *= 2;
  while (ib > 1 && staged_smem_bytes(ib, kStagedThreads / ib, g.max_es, g.max_nv, t0) > budget)
    ib /= 2;
  const size_t fixed = staged_smem_bytes(ib, 0, g.max_es, g.max_nv, t0);
  const size_t per = 4 * (size_t)(ib + g.max_nv);
  int64_t tk = fixed < budget ? (int64_t)((budget - fixed) / per) : 1;
  tk = std::max<int64_t>(1, std::min<int64_t>(tk, std::max<int64_t>(g.max_cfg, 1)));
  return StagedShape{ib, (int)tk, staged_smem_bytes(ib, (int)tk, g.max_es, g.max_nv, t0)};
}

// The built-in rule between the two generic Enum kernels (the tuner times both on run()): the
// staged one once a factor's table holds more than 128 (config, variable) entries or its
// per-thread arrays would exceed 32 edge states. Measured per iteration (T = 0, B = 1 / 32 / 128):
// 3,000 ternary 10-state factors with all 1,000 configs 0.80 / 0.69 / 1.60 ms per-thread against
// 0.06 / 0.37 / 1.35 ms staged; 20,000 8-ary binary factors with 128 configs 0.31 / 0.67 / 2.46
// against 0.22 / 0.40 / 1.52; 50,000 ternary 3-state factors with 14 configs 0.03 / 0.19 / 0.77
// against 0.28 / 0.41 / 1.59 (a CTA per factor is too coarse for them).
bool staged_rule(const EnumGeneric& g) { return g.max_cfg * g.max_nv > 128 || g.max_es > 32; }

template <bool T0, class C>
cudaError_t launch_staged(cudaStream_t s, const Plan& p, const EnumGeneric& g, const C& c,
                          int64_t B, float t, unsigned* deltas) {
  static const cudaError_t attr = cudaFuncSetAttribute(
      enum_staged_kernel<T0, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
  if (attr != cudaSuccess) return attr;
  const StagedShape sh = staged_shape(g, B, T0);
  const int64_t groups = (B + sh.ib - 1) / sh.ib;
  const dim3 grid((unsigned)groups, (unsigned)std::min<int64_t>(g.count, 65535));
  launch_pdl_smem(s, grid, dim3(kStagedThreads), sh.smem, enum_staged_kernel<T0, C>, c, dev(g), B,
                  sh.ib, sh.tk, g.max_es, g.max_nv, t, deltas);
  return cudaSuccess;
}

// variant: 0 = per-thread kernel, 1 = staged kernel (contexts with HasStaged), -1 = the rule;
// the debug knob PGBP_DEBUG_ENUM_KERNEL overrides both.
template <bool T0, class C>
void launch_enum_generic(cudaStream_t s, const Plan& p, const C& c, int64_t B, float t,
                         unsigned* deltas, const EnumGeneric* set = nullptr, int variant = -1) {
  const EnumGeneric& g = set != nullptr ? *set : p.enum_generic;
  if (g.count == 0) return;
  ProfileScope ps(kProfEnumGeneric, s);
  if constexpr (HasStaged<C>::value) {
    const int knob = debug_knobs().enum_kernel;
    const bool staged = knob == 1 ? false : knob == 2 ? true : variant >= 0 ? variant == 1
                                                                             : staged_rule(g);
    if (staged && launch_staged<T0>(s, p, g, c, B, t, deltas) == cudaSuccess) return;
  }
  const Launch2 l = launch2(g.count, B, p.sm_count);
  const EnumGenericDev d = dev(g);
  if (g.max_es <= 8) {
    launch_pdl(s, l.grid, l.block, enum_generic_kernel<8, T0, C>, c, d, B, t, deltas);
  } else if (g.max_es <= 32) {
    launch_pdl(s, l.grid, l.block, enum_generic_kernel<32, T0, C>, c, d, B, t, deltas);
  } else if (g.max_es <= 128) {
    launch_pdl(s, l.grid, l.block, enum_generic_kernel<128, T0, C>, c, d, B, t, deltas);
  } else {
    launch_pdl(s, l.grid, l.block, enum_generic_kernel<512, T0, C>, c, d, B, t, deltas);
  }
}

// Plan::unary2 of the multi-kernel iteration: 4 instances per thread when B allows it and that
// still leaves >= 16 warps per SM.
template <bool T0>
void launch_unary2(cudaStream_t s, const Plan& p, const Fused& c, int64_t B, float t,
                   unsigned* deltas) {
  if (p.unary2.count == 0) return;
  ProfileScope ps(kProfEnumGeneric, s);
  const Unary2Dev d{p.unary2.rec, p.unary2.count};
  if (B % 4 == 0 && p.unary2.count * (B / 4) >= (int64_t)p.sm_count * 16 * 32) {
    const Launch2 l = launch2_x4(p.unary2.count, B, p.sm_count);
    launch_pdl(s, l.grid, l.block, unary2_x4_kernel<T0>, c, d, t, deltas);
  } else {
    const Launch2 l = launch2(p.unary2.count, B, p.sm_count);
    launch_pdl(s, l.grid, l.block, unary2_kernel<T0>, c, d, t, deltas);
  }
}

// variant: 0 a thread per (factor, instance), 1 a warp per (factor, instance), -1 the built-in
// rule (a warp when factors have 8 parents or more on average)
template <bool T0, class C>
void launch_logical(cudaStream_t s, const Plan& p, int which, const C& c, int64_t B, float t,
                    bool low_t, int normalize, unsigned* deltas, int variant = -1) {
  const LogicalSet& g = p.logical[which];
  if (g.count == 0) return;
  ProfileScope ps(which == 0 ? kProfOr : kProfAnd, s);
  const bool warp = variant >= 0 ? variant == 1 : g.num_parents >= 8 * g.count;
  if (warp) {  // many parents per factor: a warp per factor
    const int64_t warps = g.count * B;
    const int64_t blocks = std::max<int64_t>(
        1, std::min<int64_t>((warps + 7) / 8, (int64_t)p.sm_count * 16));
    launch_pdl(s, dim3((unsigned)blocks), dim3(256), logical_warp_kernel<T0, C>, c, dev(g), B, t,
               low_t, normalize, deltas);
    return;
  }
  const Launch2 l = launch2(g.count, B, p.sm_count);
  launch_pdl(s, l.grid, l.block, logical_kernel<T0, C>, c, dev(g), B, t, low_t, normalize, deltas);
}

template <bool T0, class C>
void launch_pool(cudaStream_t s, const Plan& p, const C& c, int64_t B, float t, int normalize,
                 unsigned* deltas) {
  const PoolSet& g = p.pool;
  if (g.count == 0) return;
  ProfileScope ps(kProfPool, s);
  const Launch2 l = launch2(g.count, B, p.sm_count);
  launch_pdl(s, l.grid, l.block, pool_kernel<T0, C>, c, dev(g), B, t, normalize, deltas);
}

VarsumDev dev(const VarsumSet& v) {
  return VarsumDev{v.vs, v.off, v.slots, v.run_off, v.runs, v.count};
}

// vb_variant: 0 one instance per thread for the binary variables, 1 four (B % 4 == 0), -1 the
// built-in rule; vo_variant: the other variables' sums per state unit (0) or by variable (1, when
// built; -1 the rule: by variable when built)
void launch_varsum(cudaStream_t s, const Plan& p, int64_t B, const float* cur, const float* ev,
                   int64_t evs, int64_t evb, float* vsum, int vb_variant = -1,
                   int vo_variant = -1) {
  ProfileScope ps(kProfVarsum, s);
  const VarsumSet& vb = p.varsum_binary;
  // 4 instances per thread only when that still leaves >= 16 warps per SM: the per-variable sums
  // are serial chains, so latency is hidden by warps, not by the work inside one thread.
  // vb_variant: 0 one instance per thread, 1 four, 2 two (B % 2 == 0); -1 the rule.
  const bool x4 = B % 4 == 0 && (vb_variant >= 0 ? vb_variant == 1
                                                 : vb.count * (B / 4) >= (int64_t)p.sm_count * 16 * 32);
  if (vb.count > 0 && vb_variant == 2 && B % 2 == 0) {
    const Launch2 l = launch2(vb.count, B / 2, p.sm_count);
    launch_pdl(s, l.grid, l.block, varsum_binary_x2_kernel, dev(vb), vb.use_runs, cur, ev, evs, evb,
               vsum, B);
  } else if (vb.count > 0 && x4) {
    const Launch2 l = launch2_x4(vb.count, B, p.sm_count);
    launch_pdl(s, l.grid, l.block, varsum_binary_x4_kernel, dev(vb), vb.use_runs, cur, ev, evs, evb,
               vsum, B);
  } else if (vb.count > 0) {
    const Launch2 l = launch2(vb.count, B, p.sm_count);
    launch_pdl(s, l.grid, l.block, varsum_binary_kernel, dev(vb), vb.use_runs, cur, ev, evs, evb,
               vsum, B);
  }
  const VarsumSet& vo = p.varsum_other;
  if (vo.byvar_groups > 0 && vo_variant != 0) {
    const Launch2 l = launch2(vo.byvar_units, B, p.sm_count);
    launch_pdl(s, l.grid, l.block, varsum_byvar_kernel, vo.byvar_grp, vo.byvar_groups,
               vo.byvar_units, vo.byvar_vs0, vo.byvar_eoff, vo.byvar_eslot, cur, ev, evs, evb, vsum,
               B);
  } else if (vo.count > 0) {
    const Launch2 l = launch2(vo.count, B, p.sm_count);
    launch_pdl(s, l.grid, l.block, varsum_other_kernel, dev(vo), vo.use_runs, cur, ev, evs, evb,
               vsum, B);
  }
}

// One dense pairwise bucket of one iteration. variant: for 2 x 2 tables 0 one instance per
// thread, 1 four (B % 4 == 0); for shared K x K tables at temperature > 0 (tables != null) 0 the
// direct kernel, 1 the exp-domain tensor-core kernel; -1 the built-in rule.
template <bool T0>
void launch_bucket(cudaStream_t s, const Plan& p, const PairwiseBucket& q, const Fused& c,
                   int64_t B, float t, unsigned* d, const float* tables, int variant) {
  if (!T0 && tables != nullptr && expgemm_eligible(q) && variant != 0) {
    expgemm_iterate(p, q, s, B, c.cur, c.nxt, c.vsum, c.lp, tables, c.d, c.omd, t, d);
    return;
  }
  // 4 instances per thread only when that still leaves >= 16 warps per SM; below that the
  // kernel is latency-bound and one instance per thread keeps 4x more warps in flight
  const bool x4 = q.n1 == 2 && q.n2 == 2 && B % 4 == 0 && q.count > 0 &&
                  (variant >= 0 ? variant == 1 : q.count * (B / 4) >= (int64_t)p.sm_count * 16 * 32);
  if (x4) {
    ProfileScope ps(kProfPairwise, s);
    const Launch2 l = launch2_x4(q.count, B, p.sm_count);
    launch_pdl(s, l.grid, l.block, pairwise22_x4_kernel<T0>, c, dev(q), t, d);
  } else {
    launch_pairwise<T0>(s, p, q, c, B, t, d);
  }
}

int num_sites(const Plan& p) { return num_tune_sites(p); }

// The generic Enum set the multi-kernel iteration launches (the unary binary factors, when
// present, run on their own kernel).
const EnumGeneric& iterate_generic(const Plan& p) {
  return p.unary2.count > 0 ? p.enum_generic_rest : p.enum_generic;
}

// sites: the tuned variant per launch site (tuned_sites' layout) or null for the built-in rules
template <bool T0>
void iterate(cudaStream_t s, const Plan& p, int64_t B, Fused c, float t, bool low_t, int64_t iters,
             float* msgs0, float* msgs1, const float* ev, int64_t evs, int64_t evb,
             unsigned* dacc, const float* gemm_tables, const int* sites) {
  const int nq = (int)p.pairwise.size();
  auto site = [&](int i) { return sites != nullptr ? sites[i] : -1; };
  for (int64_t it = 0; it < iters; ++it) {
    float* cur = (it & 1) ? msgs1 : msgs0;
    float* nxt = (it & 1) ? msgs0 : msgs1;
    c.cur = cur;
    c.nxt = nxt;
    unsigned* d = dacc + it * B;
    launch_varsum(s, p, B, cur, ev, evs, evb, const_cast<float*>(c.vsum), site(0), site(1));
    const float* tables = gemm_tables;
    for (int qi = 0; qi < nq; ++qi) {
      const PairwiseBucket& q = p.pairwise[qi];
      launch_bucket<T0>(s, p, q, c, B, t, d, tables, site(2 + qi));
      if (tables != nullptr) tables += q.gemm_floats;
    }
    if (p.unary2.count > 0) launch_unary2<T0>(s, p, c, B, t, d);
    launch_enum_generic<T0>(s, p, c, B, t, d, &iterate_generic(p), site(4 + nq));
    launch_logical<T0>(s, p, 0, c, B, t, low_t, 1, d, site(2 + nq));
    launch_logical<T0>(s, p, 1, c, B, t, low_t, 1, d, site(3 + nq));
    launch_pool<T0>(s, p, c, B, t, 1, d);
  }
}

// Variant per launch site of the multi-kernel path for (batch, temperature == 0): the cached
// choice, else each site with more than one bit-identical variant timed on the run's own buffers
// (three launches per variant after one warm-up), so the choice never changes a result. The trials write the next-message buffer, the variable sums and the first
// row of residuals, which the caller resets. Inside a stream capture nothing is timed and the
// built-in rules apply (null).
template <bool T0>
const int* tune_sites(const Plan& p, cudaStream_t s, int64_t B, Fused c, float t, bool low_t,
                      const float* ev, int64_t evs, int64_t evb, unsigned* dacc,
                      const float* gemm_tables, bool* tuned_now) {
  *tuned_now = false;
  const std::pair<int64_t, bool> key{B, T0};
  {
    std::lock_guard<std::mutex> lock(p.tune_mu);
    auto it = p.tuned_sites.find(key);
    if (it != p.tuned_sites.end()) return it->second.data();
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return nullptr;
  }
  const int nq = (int)p.pairwise.size();
  std::vector<int> choice(num_sites(p), -1);
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  float* vsum = const_cast<float*>(c.vsum);
  // fastest of `n` variants of one site; launch(v) enqueues variant v
  auto pick = [&](int n, auto&& launch) {
    int best = -1;
    float best_ms = 0.0f;
    for (int v = 0; v < n; ++v) {
      launch(v);
      cudaEventRecord(e0, s);
      for (int r = 0; r < 3; ++r) launch(v);
      cudaEventRecord(e1, s);
      float ms = 0.0f;
      if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
        cudaGetLastError();
        continue;
      }
      if (best < 0 || ms < best_ms) {
        best = v;
        best_ms = ms;
      }
    }
    return best;
  };
  // the two variable-sum sites (binary, other) are timed with the other one's rule in place
  if (p.varsum_binary.count > 0 && B % 2 == 0) {
    // one, two and (B % 4 == 0) four instances per thread
    const int vb_variants[3] = {0, 2, 1};
    const int k = pick(B % 4 == 0 ? 3 : 2, [&](int v) {
      launch_varsum(s, p, B, c.cur, ev, evs, evb, vsum, vb_variants[v], -1);
    });
    choice[0] = k >= 0 ? vb_variants[k] : -1;
  }
  if (p.varsum_other.byvar_groups > 0 && p.varsum_other.count > 0)
    choice[1] = pick(2, [&](int v) { launch_varsum(s, p, B, c.cur, ev, evs, evb, vsum, -1, v); });
  launch_varsum(s, p, B, c.cur, ev, evs, evb, vsum);  // variable sums for the factor trials
  const float* tables = gemm_tables;
  for (int qi = 0; qi < nq; ++qi) {
    const PairwiseBucket& q = p.pairwise[qi];
    // only variants that give bit-identical results are timed: the exp-domain kernel (shared
    // tables at T > 0) agrees with the direct one within float32 accuracy, not bit for bit, so
    // it stays the rule there (a host can still choose it through pgbp_plan_tuning_set)
    const bool two = q.n1 == 2 && q.n2 == 2 && B % 4 == 0 && q.count > 0;
    if (two)
      choice[2 + qi] = pick(2, [&](int v) {
        launch_bucket<T0>(s, p, q, c, B, t, dacc, tables, v);
      });
    if (tables != nullptr) tables += q.gemm_floats;
  }
  for (int w = 0; w < 2; ++w) {
    if (p.logical[w].count > 0)
      choice[2 + nq + w] = pick(2, [&](int v) {
        launch_logical<T0>(s, p, w, c, B, t, low_t, 1, dacc, v);
      });
  }
  if (iterate_generic(p).count > 0)
    choice[4 + nq] = pick(2, [&](int v) {
      launch_enum_generic<T0>(s, p, c, B, t, dacc, &iterate_generic(p), v);
    });
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *tuned_now = true;
  std::lock_guard<std::mutex> lock(p.tune_mu);
  auto& slot = p.tuned_sites[key];
  slot = choice;
  return slot.data();
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

constexpr int64_t kSmallMaxSmem = 200 * 1024;

int small_maxes(const Plan& p) {
  const int m = p.enum_generic.max_es;
  return m <= 8 ? 8 : m <= 32 ? 32 : m <= 128 ? 128 : 512;
}

// The attribute is per kernel, shared by all plans: always allow the path's maximum.
template <bool T0, int MAXES>
cudaError_t set_small_attr(int64_t) {
  return cudaFuncSetAttribute(small_graph_kernel<T0, MAXES>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmallMaxSmem);
}

template <bool T0>
void launch_small(cudaStream_t s, const Plan& p, const SmallGraph& g, int64_t B, int64_t iters,
                  float t, bool low_t, float* msgs, unsigned* dacc) {
  const dim3 grid((unsigned)B), block(kSmallThreads);
  const size_t smem = (size_t)p.small_graph_smem;
  switch (small_maxes(p)) {
    case 8: small_graph_kernel<T0, 8><<<grid, block, smem, s>>>(g, B, iters, t, low_t, msgs, dacc); break;
    case 32: small_graph_kernel<T0, 32><<<grid, block, smem, s>>>(g, B, iters, t, low_t, msgs, dacc); break;
    case 128: small_graph_kernel<T0, 128><<<grid, block, smem, s>>>(g, B, iters, t, low_t, msgs, dacc); break;
    default: small_graph_kernel<T0, 512><<<grid, block, smem, s>>>(g, B, iters, t, low_t, msgs, dacc); break;
  }
}

template <bool T0, int MAXES>
cudaError_t launch_cluster_t(cudaStream_t s, const SmallGraph& g, int64_t B, int64_t iters, float t,
                             bool low_t, float* m0, float* m1, float* vsum, unsigned* dacc,
                             int csize) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(B * csize));
  cfg.blockDim = dim3(kSmallThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)csize;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (g.unit_of_vs != nullptr)
    return cudaLaunchKernelEx(&cfg, cluster_graph_kernel<T0, MAXES, true>, g, B, iters, t, low_t,
                              m0, m1, vsum, dacc);
  return cudaLaunchKernelEx(&cfg, cluster_graph_kernel<T0, MAXES, false>, g, B, iters, t, low_t, m0,
                            m1, vsum, dacc);
}

template <bool T0>
cudaError_t launch_cluster(cudaStream_t s, const Plan& p, const SmallGraph& g, int64_t B,
                           int64_t iters, float t, bool low_t, float* m0, float* m1, float* vsum,
                           unsigned* dacc) {
  const int cs = p.cluster_size;
  switch (small_maxes(p)) {
    case 8: return launch_cluster_t<T0, 8>(s, g, B, iters, t, low_t, m0, m1, vsum, dacc, cs);
    case 32: return launch_cluster_t<T0, 32>(s, g, B, iters, t, low_t, m0, m1, vsum, dacc, cs);
    case 128: return launch_cluster_t<T0, 128>(s, g, B, iters, t, low_t, m0, m1, vsum, dacc, cs);
    default: return launch_cluster_t<T0, 512>(s, g, B, iters, t, low_t, m0, m1, vsum, dacc, cs);
  }
}

template <bool T0, int MAXES>
cudaError_t allow_big_cluster() {
  cudaError_t e = cudaFuncSetAttribute(cluster_graph_kernel<T0, MAXES, false>,
                                       cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(cluster_graph_kernel<T0, MAXES, true>,
                             cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  return e;
}

// Largest cluster (16, else 8) that a 1024-thread CTA of the cluster kernel can be launched with.
int cluster_size_for(const Plan& p) {
  cudaError_t e = cudaSuccess;
  switch (small_maxes(p)) {
    case 8: e = allow_big_cluster<true, 8>(); if (!e) e = allow_big_cluster<false, 8>(); break;
    case 32: e = allow_big_cluster<true, 32>(); if (!e) e = allow_big_cluster<false, 32>(); break;
    case 128: e = allow_big_cluster<true, 128>(); if (!e) e = allow_big_cluster<false, 128>(); break;
    default: e = allow_big_cluster<true, 512>(); if (!e) e = allow_big_cluster<false, 512>(); break;
  }
  for (int cs : {16, 8, 4}) {
    if (cs == 16 && e != cudaSuccess) continue;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)cs);
    cfg.blockDim = dim3(kSmallThreads);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    cudaError_t q = cudaOccupancyMaxActiveClusters(&n, cluster_graph_kernel<true, 8, false>, &cfg);
    int n2 = 0;
    if (q == cudaSuccess)
      q = cudaOccupancyMaxActiveClusters(&n2, cluster_graph_kernel<false, 8, true>, &cfg);
    if (q == cudaSuccess && n > 0 && n2 > 0) return cs;
    cudaGetLastError();
  }
  cudaGetLastError();
  return 0;
}

}  // namespace

enum { kPathMulti = 0, kPathSmall = 1, kPathCluster = 2 };

// Execution path for (batch, temperature == 0): the cached choice, else the fastest of the
// eligible paths timed on a short run (the trial overwrites the run's first message buffer and
// residuals, which are then restored from the normalised inputs in `tmp`). Inside a stream
// capture nothing is timed and the single-CTA path is used.
template <class RunPath>
int choose_path(const Plan& p, cudaStream_t s, int64_t B, bool t0, bool cluster_ok,
                RunPath& run_path, const float* tmp, float* m0, unsigned* dacc, int64_t iters) {
  const std::pair<int64_t, bool> key{B, t0};
  {
    std::lock_guard<std::mutex> lock(p.tune_mu);
    auto it = p.tuned_path.find(key);
    if (it != p.tuned_path.end()) return it->second;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
    cudaGetLastError();
    return kPathSmall;
  }
  const int64_t trial = std::min<int64_t>(iters, 8);
  int best = kPathSmall;
  float best_ms = 0.0f;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    cudaGetLastError();
    return kPathSmall;
  }
  const int cands[3] = {kPathSmall, kPathCluster, kPathMulti};
  bool any = false;
  for (int cand : cands) {
    if (cand == kPathCluster && !cluster_ok) continue;
    run_path(cand, 1);  // warm the path (first launches of a kernel cost extra)
    cudaEventRecord(e0, s);
    run_path(cand, trial);
    cudaEventRecord(e1, s);
    float ms = 0.0f;
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    if (!any || ms < best_ms) {
      best = cand;
      best_ms = ms;
      any = true;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // restore the run's initial state
  if (p.num_edges > 0) {
    const Launch2 ln = launch2(p.num_edges, B, p.sm_count);
    normalize_pack_kernel<<<ln.grid, ln.block, 0, s>>>(p.edge_start, p.edge_slot, p.num_edges, tmp,
                                                        m0, B);
  }
  cudaMemsetAsync(dacc, 0, sizeof(unsigned) * (size_t)(iters * B), s);
  std::lock_guard<std::mutex> lock(p.tune_mu);
  p.tuned_path[key] = best;
  return best;
}

cudaError_t prepare_small_graph(Plan& p) {
  p.small_graph_smem = 0;
  p.cluster_size = 0;
  if (p.flags & PGBP_FLAG_NO_SMALL_GRAPH) return cudaSuccess;
  if ((int64_t)p.pairwise.size() > kSmallMaxBuckets || p.num_slots == 0) return cudaSuccess;
  p.cluster_size = cluster_size_for(p);
  const int64_t smem = (int64_t)sizeof(float) * (2 * p.num_slots + 2 * p.num_var_states);
  if (smem > kSmallMaxSmem) return cudaSuccess;
  cudaError_t e = cudaSuccess;
  switch (small_maxes(p)) {
    case 8: e = set_small_attr<true, 8>(smem); if (!e) e = set_small_attr<false, 8>(smem); break;
    case 32: e = set_small_attr<true, 32>(smem); if (!e) e = set_small_attr<false, 32>(smem); break;
    case 128: e = set_small_attr<true, 128>(smem); if (!e) e = set_small_attr<false, 128>(smem); break;
    default: e = set_small_attr<true, 512>(smem); if (!e) e = set_small_attr<false, 512>(smem); break;
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    return cudaSuccess;  // path unavailable: stay on the multi-kernel path
  }
  p.small_graph_smem = smem;
  return cudaSuccess;
}

int64_t gemm_table_floats(const Plan& p) {
  int64_t n = 0;
  for (const PairwiseBucket& q : p.pairwise) n += q.gemm_floats;
  return n;
}

size_t workspace_bytes(const Plan& p, int64_t batch, int64_t iters, bool ev_batched,
                       bool lp_batched) {
  const int64_t B = std::max<int64_t>(batch, 1);
  const int64_t it = std::max<int64_t>(iters, 1);
  size_t n = 0;
  n += 2 * align_up(sizeof(float) * (size_t)(p.num_slots * B));   // slots, ping-pong
  n += align_up(sizeof(float) * (size_t)(p.num_edge_states * B));  // edge-state-major in / out
  n += align_up(sizeof(float) * (size_t)(p.num_var_states * B));   // variable sums
  if (ev_batched) n += align_up(sizeof(float) * (size_t)(p.num_var_states * B));
  n += align_up(sizeof(float) * (size_t)(p.num_potentials * (lp_batched ? B : 1)));
  n += align_up(sizeof(unsigned) * (size_t)(it * B));
  n += align_up(sizeof(float) * (size_t)gemm_table_floats(p));
  n += align_up(sizeof(int));  // convergence count of pgbp_run_to_tolerance
  return n;
}

// first[b] = the first iteration (1-based, counted from the run's start) whose residual was below
// tol, if not already set; counts the instances still above it.
__global__ void __launch_bounds__(256) first_below_kernel(const unsigned* __restrict__ dacc,
                                                          int64_t n, int64_t B, float tol,
                                                          int64_t done, int32_t* __restrict__ first,
                                                          int* __restrict__ unconverged) {
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < B;
       b += (int64_t)gridDim.x * blockDim.x) {
    int32_t f = first[b];
    for (int64_t it = 0; f < 0 && it < n; ++it)
      if (__uint_as_float(dacc[it * B + b]) < tol) f = (int32_t)(done + it + 1);
    first[b] = f;
    if (f < 0) atomicAdd(unconverged, 1);
  }
}

// dst[b, i] = src[b * sstride + i] for a [B, n] block (sstride 0 broadcasts one row).
__global__ void __launch_bounds__(256) copy_rows_kernel(const float* __restrict__ src,
                                                        int64_t sstride, int64_t n, int64_t B,
                                                        float* __restrict__ dst) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n * B;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[(i / n) * sstride + i % n];
}

cudaError_t run_bp(const Plan& p, cudaStream_t s, int64_t B, const float* lp, int64_t lp_stride,
                   const float* ev, int64_t ev_stride, const float* msgs_in, int64_t msgs_stride,
                   float* msgs_out, float* deltas, int64_t num_iters, double damping,
                   double temperature, void* ws, size_t ws_bytes, int64_t checkpoint_every,
                   float* checkpoints, const ToleranceRun* tol_run, const Perturbation* pert) {
  const int64_t iters = std::max<int64_t>(num_iters, 1);
  // perturbed evidence differs per instance even when its base is shared
  const bool ev_b = ev_stride != 0 || pert != nullptr, lp_b = lp_stride != 0;
  char* w = static_cast<char*>(ws);
  auto take = [&](size_t bytes) {
    char* r = w;
    w += align_up(bytes);
    return r;
  };
  float* m0 = (float*)take(sizeof(float) * (size_t)(p.num_slots * B));
  float* m1 = (float*)take(sizeof(float) * (size_t)(p.num_slots * B));
  float* tmp = (float*)take(sizeof(float) * (size_t)(p.num_edge_states * B));
  float* vsum = (float*)take(sizeof(float) * (size_t)(p.num_var_states * B));
  float* evt = ev_b ? (float*)take(sizeof(float) * (size_t)(p.num_var_states * B)) : nullptr;
  float* lpc = (float*)take(sizeof(float) * (size_t)(p.num_potentials * (lp_b ? B : 1)));
  unsigned* dacc = (unsigned*)take(sizeof(unsigned) * (size_t)(iters * B));
  float* gemm_ws = (float*)take(sizeof(float) * (size_t)gemm_table_floats(p));
  int* unconverged = (int*)take(sizeof(int));
  (void)ws_bytes;
  if (tol_run != nullptr) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
      return cudaErrorStreamCaptureUnsupported;  // the stopping test reads a count on the host
  }

  // evidence and potentials in the run layout; potentials clipped (bp.py:85-87)
  const float* evp = ev;
  int64_t evs = 1, evb = 0;
  if (pert != nullptr) {
    if (p.num_var_states > 0) {
      ProfileScope ps(kProfLayout, s);
      dim3 grid((unsigned)((p.num_var_states + 31) / 32), (unsigned)((B + 31) / 32));
      to_inner_gumbel_kernel<<<grid, dim3(32, 8), 0, s>>>(
          ev, ev_stride, p.num_var_states, B, gumbel_key(pert->seed), pert->scale, evt,
          pert->evidence_out);
    }
    evp = evt;
    evs = B;
    evb = 1;
  } else if (ev_b) {
    to_inner(s, ev, ev_stride, p.num_var_states, B, evt, false, p.sm_count);
    evp = evt;
    evs = B;
    evb = 1;
  }
  int64_t lps = 1, lpb = 0;
  if (p.num_potentials > 0) {
    if (lp_b) {
      to_inner(s, lp, lp_stride, p.num_potentials, B, lpc, true, p.sm_count);
      lps = B;
      lpb = 1;
    } else {
      ProfileScope ps(kProfLayout, s);
      copy_clip_kernel<<<flat_grid(p.num_potentials, p.sm_count), 256, 0, s>>>(
          lp, p.num_potentials, lpc, 1);
    }
  }
  // initial messages, normalised and clipped (bp.py:92-96), packed into slots
  to_inner(s, msgs_in, msgs_stride, p.num_edge_states, B, tmp, false, p.sm_count);
  if (p.num_edges > 0) {
    ProfileScope ps(kProfLayout, s);
    const Launch2 ln = launch2(p.num_edges, B, p.sm_count);
    normalize_pack_kernel<<<ln.grid, ln.block, 0, s>>>(p.edge_start, p.edge_slot, p.num_edges,
                                                        tmp, m0, B);
  }
  cudaMemsetAsync(dacc, 0, sizeof(unsigned) * (size_t)(iters * B), s);

  Fused c;
  c.cur = m0;
  c.nxt = m1;
  c.vsum = vsum;
  c.lp = lpc;
  c.lps = lps;
  c.lpb = lpb;
  c.B = B;
  c.d = (float)damping;
  c.omd = (float)(1.0 - damping);
  const float t = (float)temperature;
  const bool low_t = temperature < kStabilityThre;
  const bool t0 = temperature == 0.0;
  // run-time tables of the shared-table exp-domain kernel (temperature > 0, potentials shared by
  // the batch), built once per run from the clipped potentials
  const float* gemm = nullptr;
  if (!t0 && !lp_b && gemm_table_floats(p) > 0) {
    float* tp = gemm_ws;
    for (const PairwiseBucket& q : p.pairwise) {
      if (expgemm_eligible(q)) expgemm_prepare(p, q, s, lpc, t, tp);
      tp += q.gemm_floats;
    }
    gemm = gemm_ws;
  }
  SmallGraph g;
  const bool small_ok = p.small_graph_smem > 0 && B <= 65535;
  const bool cluster_ok = small_ok && p.cluster_size > 0;
  if (small_ok) {
    g.n_pw = (int)p.pairwise.size();
    for (int q = 0; q < g.n_pw; ++q) g.pw[q] = dev(p.pairwise[q]);
    g.eg = dev(p.enum_generic);
    g.lg[0] = dev(p.logical[0]);
    g.lg[1] = dev(p.logical[1]);
    g.pool = dev(p.pool);
    g.vb = dev(p.varsum_binary);
    g.vo = dev(p.varsum_other);
    g.vb_runs = p.varsum_binary.use_runs;
    g.vo_runs = p.varsum_other.use_runs;
    g.unit_of_vs = p.inline_vsum ? p.vb_unit_of_vs : nullptr;
    g.num_slots = p.num_slots;
    g.num_var_states = p.num_var_states;
    g.ev = evp;
    g.evs = evs;
    g.evb = evb;
    g.lp = lpc;
    g.lps = lps;
    g.lpb = lpb;
    g.d = c.d;
    g.omd = c.omd;
  }
  // kernel variants of the multi-kernel path (null: built-in rules until tuned)
  const int* sites = nullptr;
  // run `n` iterations on execution path `path`; returns the buffer holding the result
  auto run_path = [&](int path, int64_t n) -> float* {
    if (path == kPathSmall) {
      ProfileScope ps(kProfSmallGraph, s);
      if (t0) launch_small<true>(s, p, g, B, n, t, low_t, m0, dacc);
      else launch_small<false>(s, p, g, B, n, t, low_t, m0, dacc);
      return m0;
    }
    if (path == kPathCluster) {
      ProfileScope ps(kProfSmallGraph, s);
      if (t0) launch_cluster<true>(s, p, g, B, n, t, low_t, m0, m1, vsum, dacc);
      else launch_cluster<false>(s, p, g, B, n, t, low_t, m0, m1, vsum, dacc);
      return (n & 1) ? m1 : m0;
    }
    if (t0) iterate<true>(s, p, B, c, t, low_t, n, m0, m1, evp, evs, evb, dacc, nullptr, sites);
    else iterate<false>(s, p, B, c, t, low_t, n, m0, m1, evp, evs, evb, dacc, gemm, sites);
    return (n & 1) ? m1 : m0;
  };
  int path = kPathMulti;
  if (small_ok) {
    if (p.flags & PGBP_FLAG_PATH_SMALL) {
      path = kPathSmall;
    } else if ((p.flags & PGBP_FLAG_PATH_CLUSTER) && cluster_ok) {
      path = kPathCluster;
    } else if (p.flags & PGBP_FLAG_PATH_MULTI) {
      path = kPathMulti;
    } else {
      path = choose_path(p, s, B, t0, cluster_ok, run_path, tmp, m0, dacc, iters);
    }
  }
  if (path == kPathMulti) {
    bool tuned_now = false;
    sites = t0 ? tune_sites<true>(p, s, B, c, t, low_t, evp, evs, evb, dacc, nullptr, &tuned_now)
               : tune_sites<false>(p, s, B, c, t, low_t, evp, evs, evb, dacc, gemm, &tuned_now);
    if (tuned_now) cudaMemsetAsync(dacc, 0, sizeof(unsigned) * (size_t)(iters * B), s);
  }
  // caller-layout messages of the run buffer `src` into dst [B, E_s]
  auto write_out = [&](const float* src, float* dst) {
    if (p.num_edges > 0) {
      ProfileScope ps(kProfLayout, s);
      const Launch2 ln = launch2(p.num_edges, B, p.sm_count);
      unpack_kernel<<<ln.grid, ln.block, 0, s>>>(p.edge_start, p.edge_slot, p.num_edges, src, tmp,
                                                  B);
    }
    to_outer(s, tmp, p.num_edge_states, B, dst, p.num_edge_states, p.sm_count);
  };
  // With checkpoints, the iterations run in chunks of k and the messages after every k
  // iterations are written out (checkpoint 0 is the input as given). A chunk continues from the
  // buffer the previous one ended in, so the messages and residuals are those of one long run.
  const int64_t k = checkpoints ? std::max<int64_t>(1, std::min(checkpoint_every, iters)) : iters;
  if (checkpoints) {
    ProfileScope ps(kProfLayout, s);
    copy_rows_kernel<<<flat_grid(p.num_edge_states * B, p.sm_count), 256, 0, s>>>(
        msgs_in, msgs_stride, p.num_edge_states, B, checkpoints);
  }
  if (tol_run != nullptr) {
    // chunks of `iters` iterations until every instance's residual fell below the tolerance
    cudaMemsetAsync(tol_run->first_below, 0xff, sizeof(int32_t) * (size_t)B, s);
    int64_t done = 0;
    while (done < tol_run->max_iters) {
      const int64_t n = std::min(iters, tol_run->max_iters - done);
      cudaMemsetAsync(dacc, 0, sizeof(unsigned) * (size_t)(n * B), s);
      float* fin = run_path(path, n);
      if (fin != m0) std::swap(m0, m1);
      cudaMemsetAsync(unconverged, 0, sizeof(int), s);
      {
        ProfileScope ps(kProfLayout, s);
        first_below_kernel<<<flat_grid(B, p.sm_count), 256, 0, s>>>(
            dacc, n, B, (float)tol_run->tol, done, tol_run->first_below, unconverged);
      }
      done += n;
      int left = 0;
      cudaError_t e = cudaMemcpyAsync(&left, unconverged, sizeof(int), cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return e;
      if (left == 0) break;
    }
    *tol_run->iters_run = done;
    write_out(m0, msgs_out);
    return cudaGetLastError();
  }
  unsigned* const dacc0 = dacc;
  float* fin = m0;
  for (int64_t done = 0; done < iters;) {
    const int64_t n = std::min(k, iters - done);
    dacc = dacc0 + done * B;
    fin = run_path(path, n);
    done += n;
    if (done < iters) {
      write_out(fin, checkpoints + (done / k) * B * p.num_edge_states);
      if (fin != m0) std::swap(m0, m1);
    }
  }
  dacc = dacc0;
  write_out(fin, msgs_out);
  if (deltas != nullptr) {
    ProfileScope ps(kProfLayout, s);
    deltas_out_kernel<<<flat_grid(iters * B, p.sm_count), 256, 0, s>>>(dacc, iters, B, deltas);
  }
  return cudaGetLastError();
}

cudaError_t factor_update(const Plan& p, cudaStream_t s, int type, int64_t B, const float* vtof,
                          int64_t vtof_stride, const float* lp, int64_t lp_stride,
                          double temperature, int normalize, float* out, int64_t out_stride) {
  Update c;
  c.vt = vtof;
  c.vts = vtof_stride;
  c.out = out;
  c.os = out_stride;
  c.base = p.msgs_range[type][0];
  c.lp = lp;
  c.lpb = lp_stride;
  c.lpbase = p.potentials_range[type][0];
  const float t = (float)temperature;
  const bool low_t = temperature < kStabilityThre;
  const bool t0 = temperature == 0.0;
  if (type == PGBP_ENUM) {
    for (const PairwiseBucket& q : p.pairwise) {
      if (t0) launch_pairwise<true>(s, p, q, c, B, t, nullptr);
      else launch_pairwise<false>(s, p, q, c, B, t, nullptr);
    }
    if (t0) launch_enum_generic<true>(s, p, c, B, t, nullptr);
    else launch_enum_generic<false>(s, p, c, B, t, nullptr);
  } else if (type == PGBP_OR || type == PGBP_AND) {
    if (t0) launch_logical<true>(s, p, type - 1, c, B, t, low_t, normalize, nullptr);
    else launch_logical<false>(s, p, type - 1, c, B, t, low_t, normalize, nullptr);
  } else {
    if (t0) launch_pool<true>(s, p, c, B, t, normalize, nullptr);
    else launch_pool<false>(s, p, c, B, t, normalize, nullptr);
  }
  return cudaGetLastError();
}

cudaError_t beliefs(const Plan& p, cudaStream_t s, int64_t B, const float* ev, int64_t ev_stride,
                    const float* msgs, int64_t msgs_stride, float* out) {
  if (p.num_var_states == 0) return cudaSuccess;
  ProfileScope ps(kProfReadout, s);
  const Launch2 l = launch2(p.num_var_states, B, p.sm_count);
  beliefs_kernel<<<l.grid, l.block, 0, s>>>(p.vs_off, p.vs_edges, p.num_var_states, msgs,
                                            msgs_stride, ev, ev_stride, out, B);
  return cudaGetLastError();
}

cudaError_t decode(const Plan& p, cudaStream_t s, int64_t B, const float* bel, int64_t stride,
                   int32_t* map) {
  if (p.num_variables == 0) return cudaSuccess;
  ProfileScope ps(kProfReadout, s);
  decode_kernel<<<flat_grid(p.num_variables * B, p.sm_count), 256, 0, s>>>(
      p.var_off, 0, p.num_variables, bel, stride, map, B);
  return cudaGetLastError();
}

cudaError_t marginals(const Plan& p, cudaStream_t s, int64_t B, const float* bel, int64_t stride,
                      float* out) {
  if (p.num_variables == 0) return cudaSuccess;
  ProfileScope ps(kProfReadout, s);
  marginals_kernel<<<flat_grid(p.num_variables * B, p.sm_count), 256, 0, s>>>(
      p.var_off, 0, p.num_variables, bel, stride, out, B, p.num_var_states);
  return cudaGetLastError();
}

cudaError_t gumbel(cudaStream_t s, uint64_t seed, int64_t count, float* out, int sm_count) {
  if (count == 0) return cudaSuccess;
  ProfileScope ps(kProfLayout, s);
  gumbel_fill_kernel<<<flat_grid(count, sm_count), 256, 0, s>>>(gumbel_key(seed), 0, count, out);
  return cudaGetLastError();
}

cudaError_t rows_argmax(cudaStream_t s, int64_t rows, int64_t k, const float* in, int32_t* out,
                        int sm_count) {
  if (rows == 0) return cudaSuccess;
  ProfileScope ps(kProfReadout, s);
  decode_kernel<<<flat_grid(rows, sm_count), 256, 0, s>>>(nullptr, k, rows, in, 0, out, 1);
  return cudaGetLastError();
}

cudaError_t rows_softmax(cudaStream_t s, int64_t rows, int64_t k, const float* in, float* out,
                         int sm_count) {
  if (rows == 0) return cudaSuccess;
  ProfileScope ps(kProfReadout, s);
  marginals_kernel<<<flat_grid(rows, sm_count), 256, 0, s>>>(nullptr, k, rows, in, 0, out, 1, 0);
  return cudaGetLastError();
}

// ============================================================================= SDLP
// The smooth dual of the LP relaxation of MAP (pgmax/infer/dual_lp.py:60-463). One objective
// evaluation (smooth_dual_objval_and_grad, dual_lp.py:65-236):
//   var_sums = evidence.at[var_states_for_edge_states].add(ftov)
//   per variable: softmax and T-logsumexp of var_sums (T = 0: last argmax indicator and max)
//   bp = FAC_TO_VAR_UPDATES[type](-ftov, lp, T, normalize=False)            (the factor kernels)
//   per edge: softmax and T-logsumexp of bp - ftov over its states (T = 0: -1 at the last argmax
//   and the max); grad = softmax_var[var_states_for_edge_states] - softmax_edge
//   objval = sum_variables lse + sum_factors max over the factor's edges of the edge lse
// and one step of run_with_objvals (dual_lp.py:285-307):
//   eta' = ftov - step * grad (step = lr, or lr / sqrt(it + 1) at T = 0)
//   ftov' = eta' + (it + 1) / (it + 4) * (eta' - eta)
// Layout during a run: every per-state array is [n][B] (the instance index fastest), so the
// lanes of a warp, which run one unit for consecutive instances, read consecutive words; caller
// arrays [B][n] are transposed once on entry and exit. The per-edge part runs in the store
// epilogue of the factor kernels (the Sdlp access class): a step reads each message, eta and the
// edge's variable softmax once and writes the message, eta and the edge's logsumexp once.
// float32 throughout, operations in the reference's order (label scatters in index order); the
// objective sums are double, reduced in a fixed order (per block over its unit lanes, then per
// instance over the blocks).
namespace {

struct Sdlp {
  const float* __restrict__ cur;   // dual messages [E_s][B]
  const float* __restrict__ lp;
  int64_t lps, lpb;                // potential k of instance b at lp[k * lps + b * lpb]
  const float* __restrict__ svar;  // variable softmax (T > 0) / argmax indicator (T = 0) [N_vs][B]
  float* __restrict__ lse;         // edge logsumexp (max at T = 0) at the edge's first slot [S][B]
  float* __restrict__ nxt;         // step: next messages [E_s][B]; null = no step
  float* __restrict__ eta;         // step: the sequence eta [E_s][B], in place
  float* __restrict__ upd;         // optional: factor updates, caller layout [B][E_s]
  float* __restrict__ grad;        // optional: gradient, caller layout [B][E_s]
  int64_t B, n_es;
  float t, rt, step, coef;  // rt = 1 / t (T > 0)
  bool t0;

  __device__ __forceinline__ float pot(int64_t k, int64_t b) const {
    return __ldg(lp + k * lps + b * lpb);
  }

  __device__ __forceinline__ void load(const EdgeRef& r, int k, int64_t b, float* old,
                                       float* vt) const {
    for (int i = 0; i < k; ++i) {
      old[i] = cur[(r.es0 + i) * B + b];
      vt[i] = -old[i];
    }
  }

  // The epilogue of one edge with data d[i] = bp - ftov and e[i] = t exp((d[i] - m) / t)
  // materialised once (edges of up to kMaxK states; registers once the factor kernel's state count
  // is a compile-time constant). At T > 0 the divisions by t and by the sum are products with the
  // reciprocal (within 2 ulp of the quotient; T > 0 is compared within a tolerance, T = 0 stays
  // bit-exact and divides nothing).
  static constexpr int kMaxK = 64;

  template <class F>
  __device__ __forceinline__ void store(const EdgeRef& r, int k, const float* old, F outv,
                                        int64_t b, float& dmax) const {
    if (k > kMaxK) {
      store_long(r, k, old, outv, b, dmax);
      return;
    }
    float d[kMaxK], e[kMaxK];
    float m = -INFINITY;
    for (int i = 0; i < k; ++i) {
      d[i] = outv(i) - old[i];
      m = fmaxp(m, d[i]);
    }
    int arg = k - 1;
    float sum = 0.0f;
    if (t0) {
      for (int i = 0; i < k; ++i) arg = d[i] == m ? i : arg;
    } else {
      for (int i = 0; i < k; ++i) {
        e[i] = t * expf((d[i] - m) * rt);
        sum = sum + e[i];
      }
    }
    lse[r.slot * B + b] = t0 ? m : m + t * logf(sum * rt);
    const float rs = t0 ? 0.0f : 1.0f / sum;
    for (int i = 0; i < k; ++i) {
      const int64_t at = (r.es0 + i) * B + b;
      const float sv = svar[(r.vs0 + i) * B + b];
      const float g = t0 ? sv + (i == arg ? -1.0f : 0.0f) : sv - e[i] * rs;
      if (upd != nullptr) upd[b * n_es + r.es0 + i] = outv(i);
      if (grad != nullptr) grad[b * n_es + r.es0 + i] = g;
      if (nxt != nullptr) {
        const float en = old[i] - step * g;
        nxt[at] = en + coef * (en - eta[at]);
        eta[at] = en;
      }
    }
  }

  // Edges of more than kMaxK states: the same arithmetic, recomputed instead of kept.
  template <class F>
  __device__ __noinline__ void store_long(const EdgeRef& r, int k, const float* old, F outv,
                                          int64_t b, float&) const {
    float m = -INFINITY;
    for (int i = 0; i < k; ++i) m = fmaxp(m, outv(i) - old[i]);
    int arg = k - 1;  // the last state attaining the max (the last state when none does)
    float sum = 0.0f;
    if (t0) {
      for (int i = 0; i < k; ++i) arg = (outv(i) - old[i] == m) ? i : arg;
    } else {
      for (int i = 0; i < k; ++i) sum = sum + t * expf((outv(i) - old[i] - m) * rt);
    }
    lse[r.slot * B + b] = t0 ? m : m + t * logf(sum * rt);
    const float rs = t0 ? 0.0f : 1.0f / sum;
    for (int i = 0; i < k; ++i) {
      const int64_t at = (r.es0 + i) * B + b;
      const float sv = svar[(r.vs0 + i) * B + b];
      const float g = t0 ? sv + (i == arg ? -1.0f : 0.0f)
                         : sv - (t * expf((outv(i) - old[i] - m) * rt)) * rs;
      if (upd != nullptr) upd[b * n_es + r.es0 + i] = outv(i);
      if (grad != nullptr) grad[b * n_es + r.es0 + i] = g;
      if (nxt != nullptr) {
        const float e = old[i] - step * g;
        nxt[at] = e + coef * (e - eta[at]);
        eta[at] = e;
      }
    }
  }
};

// The SDLP pass over 2 x 2 factors is issue- and latency-bound (divisions, exp and log per state
// at T > 0): four blocks per SM (64 registers) keep more warps in flight than the three that 80
// registers allow.
template <>
struct PairwiseMinBlocks<Sdlp> {
  static constexpr int value = 4;
};

// Sums v (double) over the block's unit lanes in a fixed order; thread (tx, 0) gets the block's
// total for instance lane tx.
__device__ __forceinline__ double block_sum_units(double v) {
  __shared__ double red[256];
  const int tx = threadIdx.x, ty = threadIdx.y, bx = blockDim.x;
  red[ty * bx + tx] = v;
  __syncthreads();
  for (int s = blockDim.y / 2; s > 0; s >>= 1) {
    if (ty < s) red[ty * bx + tx] += red[(ty + s) * bx + tx];
    __syncthreads();
  }
  const double r = red[tx];
  __syncthreads();
  return r;
}

// Per (variable, instance): the variable sums (evidence plus the messages of the state's edges in
// edge order), their softmax and T-logsumexp (T = 0: indicator of the last argmax and the max).
// The block's sum of the logsumexp goes to part[blockIdx.y][b].
__global__ void __launch_bounds__(256) sdlp_var_kernel(
    const int32_t* __restrict__ var_off, int64_t nv, const int32_t* __restrict__ vs_off,
    const int32_t* __restrict__ vs_edges, const float* __restrict__ cur,
    const float* __restrict__ ev, int64_t evs, int64_t evb, float* __restrict__ vsum,
    float* __restrict__ svar, double* __restrict__ part, int64_t B, float t, bool t0) {
  const Lane l = lane(B);
  const int64_t b = l.b;
  double acc = 0.0;
  for (int64_t v = l.u0; l.valid && v < nv; v += l.ustep) {
    const int64_t s0 = var_off[v], s1 = var_off[v + 1];
    float m = -INFINITY;
    for (int64_t s = s0; s < s1; ++s) {
      float x = ev[s * evs + b * evb];
      for (int32_t k = vs_off[s]; k < vs_off[s + 1]; ++k) x = x + cur[(int64_t)vs_edges[k] * B + b];
      vsum[s * B + b] = x;
      m = fmaxp(m, x);
    }
    float obj;
    if (t0) {
      int64_t arg = s1 - 1;
      for (int64_t s = s0; s < s1; ++s) arg = vsum[s * B + b] == m ? s : arg;
      for (int64_t s = s0; s < s1; ++s) svar[s * B + b] = s == arg ? 1.0f : 0.0f;
      obj = m;
    } else {
      const float rt = 1.0f / t;
      float sum = 0.0f;
      for (int64_t s = s0; s < s1; ++s) sum = sum + t * expf((vsum[s * B + b] - m) * rt);
      const float rs = 1.0f / sum;
      for (int64_t s = s0; s < s1; ++s) svar[s * B + b] = (t * expf((vsum[s * B + b] - m) * rt)) * rs;
      obj = m + t * logf(sum * rt);
    }
    acc += (double)obj;
  }
  const double tot = block_sum_units(acc);
  if (threadIdx.y == 0 && l.valid) part[blockIdx.y * B + b] = tot;
}

// Per (factor, instance): the max over the factor's edges of the edge logsumexp (dual_lp.py:
// 221-229, a scatter-max from -inf); the block's sum goes to part[blockIdx.y][b].
__global__ void __launch_bounds__(256) sdlp_factor_kernel(
    const int32_t* __restrict__ fac_edge_off, const int32_t* __restrict__ edge_slot, int64_t nf,
    const float* __restrict__ lse, double* __restrict__ part, int64_t B) {
  const Lane l = lane(B);
  const int64_t b = l.b;
  double acc = 0.0;
  for (int64_t f = l.u0; l.valid && f < nf; f += l.ustep) {
    float m = -INFINITY;
    for (int32_t e = fac_edge_off[f]; e < fac_edge_off[f + 1]; ++e)
      m = fmaxp(m, lse[(int64_t)edge_slot[e] * B + b]);
    acc += (double)m;
  }
  const double tot = block_sum_units(acc);
  if (threadIdx.y == 0 && l.valid) part[blockIdx.y * B + b] = tot;
}

// objval[b] = (sum of the variable partials) + (sum of the factor partials), in block order.
__global__ void sdlp_objval_kernel(const double* __restrict__ pv, int64_t nv_blocks,
                                   const double* __restrict__ pf, int64_t nf_blocks, int64_t B,
                                   float* __restrict__ out, int64_t out_stride) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  double sv = 0.0, sf = 0.0;
  for (int64_t i = 0; i < nv_blocks; ++i) sv += pv[i * B + b];
  for (int64_t i = 0; i < nf_blocks; ++i) sf += pf[i * B + b];
  out[b * out_stride] = (float)(sv + sf);
}

// dst[c][r] = src[r * src_stride + c] for r < rows, c < cols (32 x 32 tiles through shared memory).
__global__ void transpose_kernel(const float* __restrict__ src, int64_t rows, int64_t cols,
                                 int64_t src_stride, float* __restrict__ dst) {
  __shared__ float tile[32][33];
  const int64_t c0 = (int64_t)blockIdx.x * 32, r0 = (int64_t)blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int64_t r = r0 + j, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[j][threadIdx.x] = src[r * src_stride + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int64_t c = c0 + j, r = r0 + threadIdx.x;
    if (r < rows && c < cols) dst[c * rows + r] = tile[threadIdx.x][j];
  }
}

void transpose(cudaStream_t s, const float* src, int64_t rows, int64_t cols, int64_t src_stride,
               float* dst) {
  if (rows <= 0 || cols <= 0) return;
  const dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
  transpose_kernel<<<grid, dim3(32, 8), 0, s>>>(src, rows, cols, src_stride, dst);
}

// edge_lse[b][e] = lse at edge e's first slot.
__global__ void sdlp_edge_lse_kernel(const int32_t* __restrict__ edge_slot, int64_t ne,
                                     const float* __restrict__ lse, float* __restrict__ out,
                                     int64_t B) {
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < ne * B;
       u += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = u / ne, e = u % ne;
    out[b * ne + e] = lse[(int64_t)edge_slot[e] * B + b];
  }
}

// Workspace: 256-byte aligned pieces.
struct SdlpWs {
  float *cur, *buf, *eta, *vsum, *svar, *lse, *ev;
  double *pv, *pf;
  int64_t nv_blocks, nf_blocks;
};

size_t align256(size_t n) { return (n + 255) / 256 * 256; }

size_t sdlp_layout(const Plan& p, int64_t B, char* base, SdlpWs* w) {
  const Launch2 lv = launch2(p.num_variables, B, p.sm_count);
  const Launch2 lf = launch2(p.num_factors, B, p.sm_count);
  const int64_t n_es = p.num_edge_states, nvs = p.num_var_states;
  const size_t fsz[7] = {(size_t)(n_es * B), (size_t)(n_es * B), (size_t)(n_es * B),
                         (size_t)(nvs * B),  (size_t)(nvs * B),  (size_t)(p.num_slots * B),
                         (size_t)(nvs * B)};
  SdlpWs tmp;
  float** dst[7] = {&tmp.cur, &tmp.buf, &tmp.eta, &tmp.vsum, &tmp.svar, &tmp.lse, &tmp.ev};
  size_t off = 0;
  for (int i = 0; i < 7; ++i) {
    *dst[i] = base ? reinterpret_cast<float*>(base + off) : nullptr;
    off += align256(std::max<size_t>(fsz[i], 1) * sizeof(float));
  }
  tmp.nv_blocks = lv.grid.y;
  tmp.nf_blocks = lf.grid.y;
  tmp.pv = base ? reinterpret_cast<double*>(base + off) : nullptr;
  off += align256((size_t)(tmp.nv_blocks * B) * sizeof(double));
  tmp.pf = base ? reinterpret_cast<double*>(base + off) : nullptr;
  off += align256((size_t)(tmp.nf_blocks * B) * sizeof(double));
  if (w) *w = tmp;
  return off;
}

// Inputs of a pass: evidence in the run layout [N_vs][B] (or shared), potentials as given.
struct SdlpIn {
  const float* ev;
  int64_t evs, evb;
  const float* lp;
  int64_t lps, lpb;
};

SdlpIn sdlp_inputs(const Plan& p, cudaStream_t s, int64_t B, const float* lp, int64_t lp_stride,
                   const float* ev, int64_t ev_stride, const SdlpWs& w) {
  SdlpIn in;
  if (ev_stride == 0 || B == 1) {
    in.ev = ev;
    in.evs = 1;
    in.evb = 0;
  } else {
    transpose(s, ev, B, p.num_var_states, ev_stride, w.ev);
    in.ev = w.ev;
    in.evs = B;
    in.evb = 1;
  }
  // potentials stay in the caller's layout: shared by the batch in the common case (the factor
  // kernels then read one table for every lane); per-instance potentials are read row-wise
  in.lp = lp;
  in.lps = 1;
  in.lpb = B == 1 ? 0 : lp_stride;
  return in;
}

// One objective evaluation at c.cur; with c.nxt set, also the step. objval (may be null) gets
// [B] values out_stride apart.
void sdlp_pass(const Plan& p, cudaStream_t s, int64_t B, const SdlpIn& in, const SdlpWs& w,
               const Sdlp& c, float* objval, int64_t out_stride) {
  const float t = c.t;
  const bool t0 = c.t0;
  {
    ProfileScope ps(kProfVarsum, s);
    const Launch2 l = launch2(p.num_variables, B, p.sm_count);
    sdlp_var_kernel<<<l.grid, l.block, 0, s>>>(p.var_off, p.num_variables, p.vs_off, p.vs_edges,
                                               c.cur, in.ev, in.evs, in.evb, w.vsum, w.svar, w.pv,
                                               B, t, t0);
  }
  const bool low_t = (double)t < kStabilityThre;
  for (const PairwiseBucket& q : p.pairwise) {
    if (t0) launch_pairwise<true>(s, p, q, c, B, t, nullptr);
    else launch_pairwise<false>(s, p, q, c, B, t, nullptr);
  }
  if (t0) launch_enum_generic<true>(s, p, c, B, t, nullptr);
  else launch_enum_generic<false>(s, p, c, B, t, nullptr);
  for (int which = 0; which < 2; ++which) {
    if (t0) launch_logical<true>(s, p, which, c, B, t, low_t, 0, nullptr);
    else launch_logical<false>(s, p, which, c, B, t, low_t, 0, nullptr);
  }
  if (t0) launch_pool<true>(s, p, c, B, t, 0, nullptr);
  else launch_pool<false>(s, p, c, B, t, 0, nullptr);
  ProfileScope ps(kProfReadout, s);
  if (p.num_factors > 0) {
    const Launch2 l = launch2(p.num_factors, B, p.sm_count);
    sdlp_factor_kernel<<<l.grid, l.block, 0, s>>>(p.fac_edge_off, p.edge_slot, p.num_factors,
                                                  w.lse, w.pf, B);
  }
  if (objval != nullptr)
    sdlp_objval_kernel<<<(unsigned)((B + 127) / 128), 128, 0, s>>>(
        w.pv, p.num_variables > 0 ? w.nv_blocks : 0, w.pf, p.num_factors > 0 ? w.nf_blocks : 0, B,
        objval, out_stride);
}

Sdlp sdlp_access(const Plan& p, int64_t B, const float* cur, const SdlpIn& in, const SdlpWs& w,
                 float t) {
  Sdlp c;
  c.cur = cur;
  c.lp = in.lp;
  c.lps = in.lps;
  c.lpb = in.lpb;
  c.svar = w.svar;
  c.lse = w.lse;
  c.nxt = nullptr;
  c.eta = nullptr;
  c.upd = nullptr;
  c.grad = nullptr;
  c.B = B;
  c.n_es = p.num_edge_states;
  c.t = t;
  c.rt = t > 0.0f ? 1.0f / t : 0.0f;
  c.step = 0.0f;
  c.coef = 0.0f;
  c.t0 = t == 0.0f;
  return c;
}

}  // namespace

size_t sdlp_workspace_bytes(const Plan& p, int64_t B) { return sdlp_layout(p, B, nullptr, nullptr); }

cudaError_t sdlp_objective(const Plan& p, cudaStream_t s, int64_t B, const float* lp,
                           int64_t lp_stride, const float* ev, int64_t ev_stride,
                           const float* msgs, int64_t ms, double temperature, float* objval,
                           float* grad, float* updates, float* edge_lse, void* ws) {
  SdlpWs w;
  sdlp_layout(p, B, static_cast<char*>(ws), &w);
  const SdlpIn in = sdlp_inputs(p, s, B, lp, lp_stride, ev, ev_stride, w);
  transpose(s, msgs, B, p.num_edge_states, ms, w.cur);
  Sdlp c = sdlp_access(p, B, w.cur, in, w, (float)temperature);
  c.grad = grad;
  c.upd = updates;
  sdlp_pass(p, s, B, in, w, c, objval, 1);
  if (edge_lse != nullptr && p.num_edges > 0)
    sdlp_edge_lse_kernel<<<flat_grid(p.num_edges * B, p.sm_count), 256, 0, s>>>(
        p.edge_slot, p.num_edges, w.lse, edge_lse, B);
  return cudaGetLastError();
}

cudaError_t sdlp_run(const Plan& p, cudaStream_t s, int64_t B, const float* lp, int64_t lp_stride,
                     const float* ev, int64_t ev_stride, const float* msgs_in, int64_t ms,
                     float* msgs_out, float* objvals, int64_t iters, double temperature, double lr,
                     void* ws) {
  SdlpWs w;
  sdlp_layout(p, B, static_cast<char*>(ws), &w);
  const int64_t n = p.num_edge_states;
  if (iters <= 0) {
    if (n > 0) {
      const size_t row = (size_t)n * sizeof(float);
      cudaError_t e = cudaMemcpy2DAsync(msgs_out, row, msgs_in, (size_t)ms * sizeof(float), row,
                                        (size_t)B, cudaMemcpyDeviceToDevice, s);
      if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
  }
  const SdlpIn in = sdlp_inputs(p, s, B, lp, lp_stride, ev, ev_stride, w);
  transpose(s, msgs_in, B, n, ms, w.cur);
  if (n > 0) {
    cudaError_t e = cudaMemcpyAsync(w.eta, w.cur, (size_t)(n * B) * sizeof(float),
                                    cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
  }
  const float t = (float)temperature;
  const float lrf = (float)lr;
  float* cur = w.cur;
  float* nxt = w.buf;
  for (int64_t it = 0; it < iters; ++it) {
    Sdlp c = sdlp_access(p, B, cur, in, w, t);
    const float itf = (float)it;
    // dual_lp.py:295-305 in float32: lr * grad, or lr / sqrt(it + 1.0) * grad at T = 0
    c.step = t > 0.0f ? lrf : lrf / sqrtf(itf + 1.0f);
    c.coef = (itf + 1.0f) / (itf + 4.0f);
    c.nxt = nxt;
    c.eta = w.eta;
    sdlp_pass(p, s, B, in, w, c, objvals != nullptr ? objvals + it : nullptr, iters);
    std::swap(cur, nxt);
  }
  transpose(s, cur, n, B, B, msgs_out);
  return cudaGetLastError();
}

}  // namespace pgbp
