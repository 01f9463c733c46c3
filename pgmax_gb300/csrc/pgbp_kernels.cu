// sm_103a kernels of the loopy-BP engine.
//
// Layout in HBM during a run: messages, variable sums, evidence and (batched) potentials are stored
// "edge-major, batch innermost" - element (edge state e, instance b) at e * B + b - so the 32 lanes
// of a warp read 32 instances of the same edge state in one 128-byte transaction and every index
// (edge state -> variable state, factor -> first edge state, ...) is loaded once per warp and
// broadcast. The caller's BPArrays are [B, n] (jax.vmap layout); run() transposes them in and out
// with shared-memory tiles.
//
// One BP iteration (pgmax/infer/bp.py:98-137) is:
//   varsum_kernel    var_sums[vs] = evidence[vs] + sum of msgs over vs's edge states, serially in
//                    increasing edge-state order (the order of the reference's scatter-add,
//                    bp.py:217);
//   factor kernels   one per factor class (dense pairwise Enum, generic Enum, OR, AND, Pool). Each
//                    thread owns one (factor, instance): it forms vtof = var_sums - msgs
//                    (bp.py:218) for the factor's edge states, computes the factor-to-variable
//                    messages, and applies damping, per-edge max-normalisation, clipping at
//                    MSG_NEG_INF and the residual (bp.py:127-136) before writing - a factor owns all
//                    states of its edges, so the epilogue needs nothing from other threads.
// Everything is float32 with the reference's operation order; the build uses -fmad=false so that
// no multiply-add is contracted. At temperature 0 the engine therefore reproduces the oracle bit
// for bit; at temperature > 0 expf/logf/log1pf/expm1f differ from glibc's by an ulp or two.
#include <math.h>

#include <algorithm>

#include "pgbp_internal.h"

namespace pgbp {
namespace {

constexpr float kMsgNegInf = -1e32f;   // MSG_NEG_INF, pgmax/utils/__init__.py:26
constexpr float kLpMaxAbs = 1e6f;      // LOG_POTENTIAL_MAX_ABS, pgmax/utils/__init__.py:32
constexpr double kStabilityThre = 0.5; // TEMPERATURE_STABILITY_THRE, pgmax/factor/logical.py:33

// numpy / XLA maximum and minimum: NaN-propagating, first operand kept on ties.
__device__ __forceinline__ float fmaxp(float a, float b) { return (a >= b || a != a) ? a : b; }
__device__ __forceinline__ float fminp(float a, float b) { return (a <= b || a != a) ? a : b; }

// update_utils.py:150-166
__device__ __forceinline__ float logaddexp_t(float a, float b, float t) {
  const float mx = fmaxp(a, b);
  const float mn = fminp(a, b);
  const float w = log1pf(expf((mn - mx) / t));
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
  const float v = t * log1mexp_f((a - b) / t) + a;
  return (a >= b + eps) ? v : -INFINITY;
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
// Fused: inside run(). vtof from var sums and the current messages; outputs go through damping,
// normalisation, clipping and the residual, into the next messages.
struct Fused {
  const float* __restrict__ cur;
  float* __restrict__ nxt;
  const float* __restrict__ vsum;
  const int32_t* __restrict__ vs_of_es;
  const float* __restrict__ lp;
  int64_t lps, lpb;  // potential k of instance b at lp[k * lps + b * lpb]
  int64_t B;
  float d, omd;

  __device__ __forceinline__ float vtof(int64_t e, int64_t b) const {
    return vsum[(int64_t)__ldg(vs_of_es + e) * B + b] - cur[e * B + b];
  }
  __device__ __forceinline__ float pot(int64_t k, int64_t b) const { return __ldg(lp + k * lps + b * lpb); }

  // bp.py:127-136 for one edge whose k states start at e0; outv(i) is the new factor message.
  template <class F>
  __device__ __forceinline__ void edge(int64_t e0, int k, F outv, int64_t b, float& dmax) const {
    float m = -INFINITY;
    for (int i = 0; i < k; ++i) {
      const float o = cur[(e0 + i) * B + b];
      const float n = d * o + omd * outv(i);
      m = fmaxp(m, n);
    }
    for (int i = 0; i < k; ++i) {
      const float o = cur[(e0 + i) * B + b];
      const float n = d * o + omd * outv(i);
      const float v = fmaxp(n - m, kMsgNegInf);
      nxt[(e0 + i) * B + b] = v;
      dmax = fmaxp(dmax, fabsf(v - o));
    }
  }
};

// Update: one factor type's raw update on caller arrays [B, n_type] (FAC_TO_VAR_UPDATES call).
struct Update {
  const float* __restrict__ vt;
  int64_t vts;
  float* __restrict__ out;
  int64_t os;
  int64_t base;  // first edge state of the type
  const float* __restrict__ lp;
  int64_t lpb;   // instance stride of the potentials (0 = shared)
  int64_t lpbase;

  __device__ __forceinline__ float vtof(int64_t e, int64_t b) const { return vt[b * vts + (e - base)]; }
  __device__ __forceinline__ float pot(int64_t k, int64_t b) const { return lp[b * lpb + (k - lpbase)]; }
  template <class F>
  __device__ __forceinline__ void edge(int64_t e0, int k, F outv, int64_t b, float&) const {
    for (int i = 0; i < k; ++i) out[b * os + (e0 + i - base)] = outv(i);
  }
};

// ----------------------------------------------------------------------------- Enum factors
// pass_enum_fac_to_var_messages, pgmax/factor/enum.py:451-475, for one dense pairwise factor.
// summary(i, j) = ((0 + vtof1[i]) + vtof2[j]) + lp[i * n2 + j]; the max / sum-exp over the configs
// of an edge state run in increasing config order, the reference's scatter order.
template <int N1, int N2, bool T0, class C>
__device__ __forceinline__ void pairwise_body(const C& c, int64_t e0, int64_t k0, int n1d, int n2d,
                                              int64_t b, float t, float& dmax) {
  // N1, N2 > 0: sizes known at compile time, arrays live in registers (loops unroll).
  // N1 = N2 = 0: run-time sizes up to 64, arrays in local memory, loops not unrolled.
  constexpr int M1 = N1 > 0 ? N1 : 64;
  constexpr int M2 = N2 > 0 ? N2 : 64;
  const int n1 = N1 > 0 ? N1 : n1d;
  const int n2 = N2 > 0 ? N2 : n2d;
  float v1[M1], v2[M2], mx1[M1], mx2[M2];
  for (int i = 0; i < n1; ++i) {
    v1[i] = c.vtof(e0 + i, b);
    mx1[i] = -INFINITY;
  }
  for (int j = 0; j < n2; ++j) {
    v2[j] = c.vtof(e0 + n1 + j, b);
    mx2[j] = -INFINITY;
  }
  for (int i = 0; i < n1; ++i) {
    for (int j = 0; j < n2; ++j) {
      const float s = ((0.0f + v1[i]) + v2[j]) + c.pot(k0 + i * n2 + j, b);
      mx1[i] = fmaxp(mx1[i], s);
      mx2[j] = fmaxp(mx2[j], s);
    }
  }
  if (T0) {
    c.edge(e0, n1, [&](int i) { return mx1[i] - v1[i]; }, b, dmax);
    c.edge(e0 + n1, n2, [&](int j) { return mx2[j] - v2[j]; }, b, dmax);
  } else {
    float s1[M1], s2[M2];
    for (int i = 0; i < n1; ++i) s1[i] = 0.0f;
    for (int j = 0; j < n2; ++j) s2[j] = 0.0f;
    for (int i = 0; i < n1; ++i) {
      for (int j = 0; j < n2; ++j) {
        const float s = ((0.0f + v1[i]) + v2[j]) + c.pot(k0 + i * n2 + j, b);
        s1[i] += expf((s - mx1[i]) / t);
        s2[j] += expf((s - mx2[j]) / t);
      }
    }
    c.edge(e0, n1, [&](int i) { return (t * logf(s1[i]) + mx1[i]) - v1[i]; }, b, dmax);
    c.edge(e0 + n1, n2, [&](int j) { return (t * logf(s2[j]) + mx2[j]) - v2[j]; }, b, dmax);
  }
}

struct PairwiseDev {
  const int32_t* __restrict__ es_begin;
  const int32_t* __restrict__ cfg_begin;
  int64_t count;
  int n1, n2;
};

template <int N1, int N2, bool T0, class C>
__global__ void __launch_bounds__(256) pairwise_kernel(C c, PairwiseDev p, int64_t B, float t,
                                                       unsigned* deltas) {
  const Lane l = lane(B);
  float dmax = 0.0f;
  if (l.valid) {
    for (int64_t u = l.u0; u < p.count; u += l.ustep) {
      pairwise_body<N1, N2, T0>(c, (int64_t)__ldg(p.es_begin + u), (int64_t)__ldg(p.cfg_begin + u),
                                p.n1, p.n2, l.b, t, dmax);
    }
  }
  block_max_to(deltas, l, dmax);
}

struct EnumGenericDev {
  const int32_t* __restrict__ es_begin;
  const int32_t* __restrict__ n_es;
  const int32_t* __restrict__ edge_off;
  const int32_t* __restrict__ edge_size;
  const int32_t* __restrict__ row_begin;
  const int32_t* __restrict__ n_cfg;
  const int32_t* __restrict__ n_vars;
  const int32_t* __restrict__ cfg_begin;
  const int32_t* __restrict__ row_les;
  int64_t count;
};

// pass_enum_fac_to_var_messages (enum.py:451-475) for an arbitrary config table.
template <int MAXES, bool T0, class C>
__global__ void __launch_bounds__(256) enum_generic_kernel(C c, EnumGenericDev g, int64_t B, float t,
                                                           unsigned* deltas) {
  const Lane l = lane(B);
  float dmax = 0.0f;
  if (l.valid) {
    const int64_t b = l.b;
    for (int64_t f = l.u0; f < g.count; f += l.ustep) {
      const int64_t e0 = g.es_begin[f];
      const int n = g.n_es[f], nv = g.n_vars[f], ncfg = g.n_cfg[f];
      const int64_t rb = g.row_begin[f], k0 = g.cfg_begin[f];
      float v[MAXES], mx[MAXES], se[MAXES];
      for (int i = 0; i < n; ++i) {
        v[i] = c.vtof(e0 + i, b);
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
          for (int i = 0; i < nv; ++i) se[rows[i]] += expf((s - mx[rows[i]]) / t);
        }
      }
      int pos = 0;
      for (int j = g.edge_off[f]; j < g.edge_off[f + 1]; ++j) {
        const int k = g.edge_size[j];
        const int p0 = pos;
        if (T0) {
          c.edge(e0 + p0, k, [&](int i) { return mx[p0 + i] - v[p0 + i]; }, b, dmax);
        } else {
          c.edge(e0 + p0, k, [&](int i) { return (t * logf(se[p0 + i]) + mx[p0 + i]) - v[p0 + i]; },
                 b, dmax);
        }
        pos += k;
      }
    }
  }
  block_max_to(deltas, l, dmax);
}

// ----------------------------------------------------------------------------- OR / AND factors
struct LogicalDev {
  const int32_t* __restrict__ par_begin;
  const int32_t* __restrict__ par_es;
  const int32_t* __restrict__ child_es;
  int64_t count;
  int off;
};

// pass_logical_fac_to_var_messages, pgmax/factor/logical.py:561-779, one factor per thread.
// Factor-level sums run over the parents in order (the reference's scatter order); the argmax is
// the last parent attaining the maximum difference (update_utils.py:48-63).
template <bool T0, class C>
__global__ void __launch_bounds__(256) logical_kernel(C c, LogicalDev g, int64_t B, float t,
                                                      bool low_t, int normalize, unsigned* deltas) {
  const Lane l = lane(B);
  float dmax = 0.0f;
  const int off = g.off;
  if (l.valid) {
    const int64_t b = l.b;
    for (int64_t f = l.u0; f < g.count; f += l.ustep) {
      const int64_t p0 = g.par_begin[f], p1 = g.par_begin[f + 1];
      const int64_t ch = g.child_es[f];
      float fs_oth = 0.0f, max1 = -INFINITY, fs_x = 0.0f;
      for (int64_t i = p0; i < p1; ++i) {
        const int64_t e = g.par_es[i];
        const float vo = c.vtof(e, b), vr = c.vtof(e + off, b);
        fs_oth += vo;
        max1 = fmaxp(max1, vr - vo);
        fs_x += T0 ? fmaxp(vo, vr) : logaddexp_t(vr, vo, t);
      }
      int64_t arg = p1 - 1;
      {
        int64_t last = -1;
        for (int64_t i = p0; i < p1; ++i) {
          const int64_t e = g.par_es[i];
          if (c.vtof(e + off, b) - c.vtof(e, b) == max1) last = i;
        }
        if (last >= 0) arg = last;
      }
      float max2 = -INFINITY;
      for (int64_t i = p0; i < p1; ++i) {
        const int64_t e = g.par_es[i];
        const float dif = (i == arg) ? -INFINITY : c.vtof(e + off, b) - c.vtof(e, b);
        max2 = fmaxp(max2, dif);
      }
      const float c_rel = c.vtof(ch + off, b), c_oth = c.vtof(ch, b);
      float ch_rel;
      if (T0) {
        ch_rel = fs_x + fminp(0.0f, max1);
      } else {
        ch_rel = logminusexp_t(fs_x, fs_oth, t, 1e-4f);
        if (low_t) ch_rel = fmaxp(ch_rel, logaddexp_t(fs_oth + max1, fs_oth + max2, t));
      }
      const bool single = (p1 - p0) == 1;
      for (int64_t i = p0; i < p1; ++i) {
        const int64_t e = g.par_es[i];
        const float vo = c.vtof(e, b), vr = c.vtof(e + off, b);
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
        // the edge's two states in index order: (other, relevant) for OR, (relevant, other) for AND
        if (off > 0) {
          c.edge(e, 2, [&](int s) { return s == 0 ? oth_out : rel_out; }, b, dmax);
        } else {
          c.edge(e - 1, 2, [&](int s) { return s == 0 ? rel_out : oth_out; }, b, dmax);
        }
      }
      const float crel_out = normalize ? ch_rel - fs_oth : ch_rel;
      const float coth_out = normalize ? 0.0f : fs_oth;
      if (off > 0) {
        c.edge(ch, 2, [&](int s) { return s == 0 ? coth_out : crel_out; }, b, dmax);
      } else {
        c.edge(ch - 1, 2, [&](int s) { return s == 0 ? crel_out : coth_out; }, b, dmax);
      }
    }
  }
  block_max_to(deltas, l, dmax);
}

// ----------------------------------------------------------------------------- Pool factors
struct PoolDev {
  const int32_t* __restrict__ ch_begin;
  const int32_t* __restrict__ ch_es;
  const int32_t* __restrict__ ind_es;
  int64_t count;
};

// pass_pool_fac_to_var_messages, pgmax/factor/pool.py:328-474.
template <bool T0, class C>
__global__ void __launch_bounds__(256) pool_kernel(C c, PoolDev g, int64_t B, float t, int normalize,
                                                   unsigned* deltas) {
  const Lane l = lane(B);
  float dmax = 0.0f;
  if (l.valid) {
    const int64_t b = l.b;
    for (int64_t f = l.u0; f < g.count; f += l.ustep) {
      const int64_t p0 = g.ch_begin[f], p1 = g.ch_begin[f + 1];
      const int64_t ie = g.ind_es[f];
      float sums0 = 0.0f, max1 = -INFINITY;
      for (int64_t i = p0; i < p1; ++i) {
        const int64_t e = g.ch_es[i];
        const float z = c.vtof(e, b), o = c.vtof(e + 1, b);
        sums0 += z;
        max1 = fmaxp(max1, o - z);
      }
      int64_t arg = p1 - 1;
      {
        int64_t last = -1;
        for (int64_t i = p0; i < p1; ++i) {
          const int64_t e = g.ch_es[i];
          if (c.vtof(e + 1, b) - c.vtof(e, b) == max1) last = i;
        }
        if (last >= 0) arg = last;
      }
      const float pi_zero = c.vtof(ie, b), pi_one = c.vtof(ie + 1, b);
      const float pi_diff = pi_one - pi_zero;
      float max2 = -INFINITY, pi_mdiff, fl = 0.0f, am = 0.0f;
      if (T0) {
        for (int64_t i = p0; i < p1; ++i) {
          const int64_t e = g.ch_es[i];
          const float dif = (i == arg) ? -INFINITY : c.vtof(e + 1, b) - c.vtof(e, b);
          max2 = fmaxp(max2, dif);
        }
        pi_mdiff = max1;
      } else {
        float se = 0.0f;
        for (int64_t i = p0; i < p1; ++i) {
          const int64_t e = g.ch_es[i];
          se += expf(((c.vtof(e + 1, b) - c.vtof(e, b)) - max1) / t);
        }
        pi_mdiff = t * logf(se) + max1;
        fl = logaddexp_t(pi_mdiff, -pi_diff, t);
        // -logsumexps_with_temp of the diffs with the argmax replaced by -pi_diff (pool.py:416-425)
        float mw = -INFINITY;
        for (int64_t i = p0; i < p1; ++i) {
          const int64_t e = g.ch_es[i];
          const float w = (i == arg) ? -pi_diff : c.vtof(e + 1, b) - c.vtof(e, b);
          mw = fmaxp(mw, w);
        }
        float sw = 0.0f;
        for (int64_t i = p0; i < p1; ++i) {
          const int64_t e = g.ch_es[i];
          const float w = (i == arg) ? -pi_diff : c.vtof(e + 1, b) - c.vtof(e, b);
          sw += expf((w - mw) / t);
        }
        am = -(t * logf(sw) + mw);
      }
      const bool single = (p1 - p0) == 1;
      for (int64_t i = p0; i < p1; ++i) {
        const int64_t e = g.ch_es[i];
        const float z = c.vtof(e, b), o = c.vtof(e + 1, b);
        const float dif = o - z;
        float mdiff;
        if (T0) {
          mdiff = fminp(pi_diff, -(i == arg ? max2 : max1));
        } else {
          mdiff = (i == arg) ? am : -logminusexp_t(fl, dif, t, 1e-30f);
        }
        float ones = (sums0 + pi_one) - z;
        if (single) {
          mdiff = pi_diff;
          ones = pi_one;
        }
        const float s1 = normalize ? mdiff : ones;
        const float s0 = normalize ? 0.0f : ones - mdiff;
        c.edge(e, 2, [&](int s) { return s == 0 ? s0 : s1; }, b, dmax);
      }
      const float i1 = normalize ? pi_mdiff : sums0 + pi_mdiff;
      const float i0 = normalize ? 0.0f : sums0;
      c.edge(ie, 2, [&](int s) { return s == 0 ? i0 : i1; }, b, dmax);
    }
  }
  block_max_to(deltas, l, dmax);
}

// ----------------------------------------------------------------------------- variable sums
// var_sums = evidence.at[var_states_for_edge_states].add(msgs) (bp.py:217), serial per var state.
__global__ void __launch_bounds__(256) varsum_kernel(const int32_t* __restrict__ vs_off,
                                                     const int32_t* __restrict__ vs_edges, int64_t nvs,
                                                     const float* __restrict__ msgs,
                                                     const float* __restrict__ ev, int64_t evs,
                                                     int64_t evb, float* __restrict__ vsum, int64_t B) {
  const Lane l = lane(B);
  if (!l.valid) return;
  const int64_t b = l.b;
  for (int64_t u = l.u0; u < nvs; u += l.ustep) {
    float s = ev[u * evs + b * evb];
    const int32_t k1 = vs_off[u + 1];
    int32_t k = vs_off[u];
    for (; k + 4 <= k1; k += 4) {
      const float m0 = msgs[(int64_t)__ldg(vs_edges + k) * B + b];
      const float m1 = msgs[(int64_t)__ldg(vs_edges + k + 1) * B + b];
      const float m2 = msgs[(int64_t)__ldg(vs_edges + k + 2) * B + b];
      const float m3 = msgs[(int64_t)__ldg(vs_edges + k + 3) * B + b];
      s += m0;
      s += m1;
      s += m2;
      s += m3;
    }
    for (; k < k1; ++k) s += msgs[(int64_t)__ldg(vs_edges + k) * B + b];
    vsum[u * B + b] = s;
  }
}

// Flat beliefs from caller-layout arrays ([B, n] rows): inferer.py:218-222.
__global__ void __launch_bounds__(256) beliefs_kernel(const int32_t* __restrict__ vs_off,
                                                      const int32_t* __restrict__ vs_edges, int64_t nvs,
                                                      const float* __restrict__ msgs, int64_t ms,
                                                      const float* __restrict__ ev, int64_t evs,
                                                      float* __restrict__ out, int64_t B) {
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
// normalize_and_clip_msgs (bp.py:222-260) in the run layout, one (edge, instance) per thread.
__global__ void __launch_bounds__(256) normalize_kernel(const int32_t* __restrict__ edge_start,
                                                        int64_t ne, float* __restrict__ msgs, int64_t B) {
  const Lane l = lane(B);
  if (!l.valid) return;
  const int64_t b = l.b;
  for (int64_t u = l.u0; u < ne; u += l.ustep) {
    const int64_t s0 = edge_start[u], s1 = edge_start[u + 1];
    float m = -INFINITY;
    for (int64_t e = s0; e < s1; ++e) m = fmaxp(m, msgs[e * B + b]);
    for (int64_t e = s0; e < s1; ++e) msgs[e * B + b] = fmaxp(msgs[e * B + b] - m, kMsgNegInf);
  }
}

__device__ __forceinline__ float clip_lp(float x) { return fminp(fmaxp(x, -kLpMaxAbs), kLpMaxAbs); }

// dst[i * B + b] = src[b * sstride + i] for i < n, b < B (optionally clipped), via 32x32 tiles.
__global__ void to_inner_kernel(const float* __restrict__ src, int64_t sstride, int64_t n, int64_t B,
                                float* __restrict__ dst, int clip) {
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

// decode_map_states (inferer.py:251-264): jnp.argmax, first maximum (or first NaN) wins.
__global__ void decode_kernel(const int32_t* __restrict__ var_off, int64_t nv,
                              const float* __restrict__ bel, int64_t bs, int32_t* __restrict__ map,
                              int64_t B) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv * B;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / nv, v = i % nv;
    const int64_t s0 = var_off[v], s1 = var_off[v + 1];
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

// get_marginals (bp.py:263-288): exp(x - logsumexp(x)) per variable.
__global__ void marginals_kernel(const int32_t* __restrict__ var_off, int64_t nv,
                                 const float* __restrict__ bel, int64_t bs, float* __restrict__ out,
                                 int64_t B, int64_t nvs) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv * B;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / nv, v = i % nv;
    const int64_t s0 = var_off[v], s1 = var_off[v + 1];
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
  return PairwiseDev{q.es_begin, q.cfg_begin, q.count, q.n1, q.n2};
}
EnumGenericDev dev(const EnumGeneric& g) {
  return EnumGenericDev{g.es_begin, g.n_es,  g.edge_off, g.edge_size, g.row_begin,
                        g.n_cfg,    g.n_vars, g.cfg_begin, g.row_les,   g.count};
}
LogicalDev dev(const LogicalSet& g) {
  return LogicalDev{g.par_begin, g.par_es, g.child_es, g.count, g.off};
}
PoolDev dev(const PoolSet& g) { return PoolDev{g.ch_begin, g.ch_es, g.ind_es, g.count}; }

template <bool T0, class C>
void launch_pairwise(cudaStream_t s, const Plan& p, const PairwiseBucket& q, const C& c, int64_t B,
                     float t, unsigned* deltas) {
  if (q.count == 0) return;
  ProfileScope ps(kProfPairwise, s);
  const Launch2 l = launch2(q.count, B, p.sm_count);
  const PairwiseDev d = dev(q);
  if (q.n1 == 2 && q.n2 == 2) {
    pairwise_kernel<2, 2, T0><<<l.grid, l.block, 0, s>>>(c, d, B, t, deltas);
  } else if (q.n1 == 4 && q.n2 == 4) {
    pairwise_kernel<4, 4, T0><<<l.grid, l.block, 0, s>>>(c, d, B, t, deltas);
  } else if (q.n1 == 8 && q.n2 == 8) {
    pairwise_kernel<8, 8, T0><<<l.grid, l.block, 0, s>>>(c, d, B, t, deltas);
  } else {
    pairwise_kernel<0, 0, T0><<<l.grid, l.block, 0, s>>>(c, d, B, t, deltas);
  }
}

template <bool T0, class C>
void launch_enum_generic(cudaStream_t s, const Plan& p, const C& c, int64_t B, float t,
                         unsigned* deltas) {
  const EnumGeneric& g = p.enum_generic;
  if (g.count == 0) return;
  ProfileScope ps(kProfEnumGeneric, s);
  const Launch2 l = launch2(g.count, B, p.sm_count);
  const EnumGenericDev d = dev(g);
  if (g.max_es <= 8) {
    enum_generic_kernel<8, T0><<<l.grid, l.block, 0, s>>>(c, d, B, t, deltas);
  } else if (g.max_es <= 32) {
    enum_generic_kernel<32, T0><<<l.grid, l.block, 0, s>>>(c, d, B, t, deltas);
  } else if (g.max_es <= 128) {
    enum_generic_kernel<128, T0><<<l.grid, l.block, 0, s>>>(c, d, B, t, deltas);
  } else {
    enum_generic_kernel<512, T0><<<l.grid, l.block, 0, s>>>(c, d, B, t, deltas);
  }
}

template <bool T0, class C>
void launch_logical(cudaStream_t s, const Plan& p, int which, const C& c, int64_t B, float t,
                    bool low_t, int normalize, unsigned* deltas) {
  const LogicalSet& g = p.logical[which];
  if (g.count == 0) return;
  ProfileScope ps(which == 0 ? kProfOr : kProfAnd, s);
  const Launch2 l = launch2(g.count, B, p.sm_count);
  logical_kernel<T0><<<l.grid, l.block, 0, s>>>(c, dev(g), B, t, low_t, normalize, deltas);
}

template <bool T0, class C>
void launch_pool(cudaStream_t s, const Plan& p, const C& c, int64_t B, float t, int normalize,
                 unsigned* deltas) {
  const PoolSet& g = p.pool;
  if (g.count == 0) return;
  ProfileScope ps(kProfPool, s);
  const Launch2 l = launch2(g.count, B, p.sm_count);
  pool_kernel<T0><<<l.grid, l.block, 0, s>>>(c, dev(g), B, t, normalize, deltas);
}

template <bool T0>
void iterate(cudaStream_t s, const Plan& p, int64_t B, Fused c, float t, bool low_t, int64_t iters,
             float* msgs0, float* msgs1, const float* ev, int64_t evs, int64_t evb, unsigned* dacc) {
  const Launch2 lv = launch2(p.num_var_states, B, p.sm_count);
  for (int64_t it = 0; it < iters; ++it) {
    float* cur = (it & 1) ? msgs1 : msgs0;
    float* nxt = (it & 1) ? msgs0 : msgs1;
    c.cur = cur;
    c.nxt = nxt;
    unsigned* d = dacc + it * B;
    if (p.num_var_states > 0) {
      ProfileScope ps(kProfVarsum, s);
      varsum_kernel<<<lv.grid, lv.block, 0, s>>>(p.vs_off, p.vs_edges, p.num_var_states, cur, ev,
                                                 evs, evb, const_cast<float*>(c.vsum), B);
    }
    for (const PairwiseBucket& q : p.pairwise) launch_pairwise<T0>(s, p, q, c, B, t, d);
    launch_enum_generic<T0>(s, p, c, B, t, d);
    launch_logical<T0>(s, p, 0, c, B, t, low_t, 1, d);
    launch_logical<T0>(s, p, 1, c, B, t, low_t, 1, d);
    launch_pool<T0>(s, p, c, B, t, 1, d);
  }
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

size_t workspace_bytes(const Plan& p, int64_t batch, int64_t iters, bool ev_batched, bool lp_batched) {
  const int64_t B = std::max<int64_t>(batch, 1);
  const int64_t it = std::max<int64_t>(iters, 1);
  size_t n = 0;
  n += 2 * align_up(sizeof(float) * (size_t)(p.num_edge_states * B));
  n += align_up(sizeof(float) * (size_t)(p.num_var_states * B));
  if (ev_batched) n += align_up(sizeof(float) * (size_t)(p.num_var_states * B));
  n += align_up(sizeof(float) * (size_t)(p.num_potentials * (lp_batched ? B : 1)));
  n += align_up(sizeof(unsigned) * (size_t)(it * B));
  return n;
}

cudaError_t run_bp(const Plan& p, cudaStream_t s, int64_t B, const float* lp, int64_t lp_stride,
                   const float* ev, int64_t ev_stride, const float* msgs_in, int64_t msgs_stride,
                   float* msgs_out, float* deltas, int64_t num_iters, double damping,
                   double temperature, void* ws, size_t ws_bytes) {
  const int64_t iters = std::max<int64_t>(num_iters, 1);
  const bool ev_b = ev_stride != 0, lp_b = lp_stride != 0;
  char* w = static_cast<char*>(ws);
  auto take = [&](size_t bytes) {
    char* r = w;
    w += align_up(bytes);
    return r;
  };
  float* m0 = (float*)take(sizeof(float) * (size_t)(p.num_edge_states * B));
  float* m1 = (float*)take(sizeof(float) * (size_t)(p.num_edge_states * B));
  float* vsum = (float*)take(sizeof(float) * (size_t)(p.num_var_states * B));
  float* evt = ev_b ? (float*)take(sizeof(float) * (size_t)(p.num_var_states * B)) : nullptr;
  float* lpc = (float*)take(sizeof(float) * (size_t)(p.num_potentials * (lp_b ? B : 1)));
  unsigned* dacc = (unsigned*)take(sizeof(unsigned) * (size_t)(iters * B));
  (void)ws_bytes;

  // evidence and potentials in the run layout; potentials clipped (bp.py:85-87)
  const float* evp = ev;
  int64_t evs = 1, evb = 0;
  if (ev_b) {
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
      copy_clip_kernel<<<flat_grid(p.num_potentials, p.sm_count), 256, 0, s>>>(lp, p.num_potentials,
                                                                               lpc, 1);
    }
  }
  // initial messages, normalised and clipped (bp.py:92-96)
  to_inner(s, msgs_in, msgs_stride, p.num_edge_states, B, m0, false, p.sm_count);
  if (p.num_edges > 0) {
    ProfileScope ps(kProfLayout, s);
    const Launch2 ln = launch2(p.num_edges, B, p.sm_count);
    normalize_kernel<<<ln.grid, ln.block, 0, s>>>(p.edge_start, p.num_edges, m0, B);
  }
  cudaMemsetAsync(dacc, 0, sizeof(unsigned) * (size_t)(iters * B), s);

  Fused c;
  c.cur = m0;
  c.nxt = m1;
  c.vsum = vsum;
  c.vs_of_es = p.vs_of_es;
  c.lp = lpc;
  c.lps = lps;
  c.lpb = lpb;
  c.B = B;
  c.d = (float)damping;
  c.omd = (float)(1.0 - damping);
  const float t = (float)temperature;
  const bool low_t = temperature < kStabilityThre;
  if (temperature == 0.0) {
    iterate<true>(s, p, B, c, t, low_t, iters, m0, m1, evp, evs, evb, dacc);
  } else {
    iterate<false>(s, p, B, c, t, low_t, iters, m0, m1, evp, evs, evb, dacc);
  }
  float* fin = (iters & 1) ? m1 : m0;
  to_outer(s, fin, p.num_edge_states, B, msgs_out, p.num_edge_states, p.sm_count);
  if (deltas != nullptr) {
    ProfileScope ps(kProfLayout, s);
    deltas_out_kernel<<<flat_grid(iters * B, p.sm_count), 256, 0, s>>>(dacc, iters, B, deltas);
  }
  return cudaGetLastError();
}

cudaError_t factor_update(const Plan& p, cudaStream_t s, int type, int64_t B, const float* vtof,
                          int64_t vtof_stride, const float* lp, int64_t lp_stride, double temperature,
                          int normalize, float* out, int64_t out_stride) {
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
  beliefs_kernel<<<l.grid, l.block, 0, s>>>(p.vs_off, p.vs_edges, p.num_var_states, msgs, msgs_stride,
                                            ev, ev_stride, out, B);
  return cudaGetLastError();
}

cudaError_t decode(const Plan& p, cudaStream_t s, int64_t B, const float* bel, int64_t stride,
                   int32_t* map) {
  if (p.num_variables == 0) return cudaSuccess;
  ProfileScope ps(kProfReadout, s);
  decode_kernel<<<flat_grid(p.num_variables * B, p.sm_count), 256, 0, s>>>(p.var_off, p.num_variables,
                                                                           bel, stride, map, B);
  return cudaGetLastError();
}

cudaError_t marginals(const Plan& p, cudaStream_t s, int64_t B, const float* bel, int64_t stride,
                      float* out) {
  if (p.num_variables == 0) return cudaSuccess;
  ProfileScope ps(kProfReadout, s);
  marginals_kernel<<<flat_grid(p.num_variables * B, p.sm_count), 256, 0, s>>>(
      p.var_off, p.num_variables, bel, stride, out, B, p.num_var_states);
  return cudaGetLastError();
}

}  // namespace pgbp
