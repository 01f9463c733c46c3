// Reverse mode of the damped BP iterations of run_with_diffs (pgmax/infer/bp.py:63-155) for graphs
// of EnumFactors, OR and AND factors, at temperature > 0: the hand-written adjoint
// behind differentiable BP (gradients of a loss on the final messages with respect to the log
// potentials, the evidence and the initial messages).
//
// Forward iteration (per instance), with n = d * m + (1 - d) * f:
//   vsum[v]  = ev[v] + sum_{e in v} m[e]                                       (bp.py:191-219)
//   vtof[e]  = vsum[v(e)] - m[e]
//   s_ij     = vtof1[i] + vtof2[j] + lp_ij                                      (enum.py:451-455)
//   f1[i]    = T log sum_j exp((s_ij - M_i) / T) + M_i - vtof1[i], f2 likewise  (enum.py:456-474)
//   m'[e]    = max(n[e] - max_{e' in edge} n[e'], MSG_NEG_INF)                 (bp.py:222-260)
// Backward, given g' = dL/dm':
//   gy  = g' where n - max(n) was not clipped, else 0
//   gn  = gy - [e = first argmax of its edge] * sum over the edge of gy
//   gf  = (1 - d) gn,  gdir = d gn                               (gdir: through the damping term)
//   gs_ij = gf1[i] p1_ij + gf2[j] p2_ij,  p1_ij = softmax_j(s_ij / T), p2_ij = softmax_i(s_ij / T)
//   gvtof1[i] = sum_j gs_ij - gf1[i],  gvtof2[j] = sum_i gs_ij - gf2[j],  glp_ij += gs_ij
//   gvsum[v] = sum_{e in v} gvtof[e],  gev[v] += gvsum[v]
// For any other config table (generic EnumFactors) with config sums s_c = sum_{e in c} vtof[e] +
// lp_c and f[e] = T log sum_{c holds e} exp((s_c - M_e) / T) + M_e - vtof[e]:
//   gs_c = sum_{e in c} gf[e] p_e(c),  p_e(c) = exp((s_c - M_e) / T) / sum_{c' holds e} exp(...)
//   gvtof[e] = sum_{c holds e} gs_c - gf[e],  glp_c += gs_c
// (the pairwise formulas are this with c = (i, j)).
// OR / AND factors (logical.py:645-779, normalize=True) are differentiated through their closed
// form: parent differences, the factor sums FO = sum of the other-state messages and FX = sum of
// logaddexp(rel, other), logaddexp / logminusexp of those, the temperature < 0.5 lower bounds
// with the top two parent differences, and the single-parent rule. At logminusexp's eps cutoff
// (which returns the constant -inf) and through a maximum the gradient follows the selected
// branch; the derivative of logaddexp_t(a, b) is exp((a - l) / t), that of logminusexp_t(a, b)
// is 1 / (1 - e) and -e / (1 - e) with e = exp((b - a) / t).
//   g[e] (= dL/dm) = gdir[e] + gvsum[v(e)] - gvtof[e]
// g is never stored: the next (earlier) step's factor kernel reads gdir, gvsum and gvtof of the
// step after it and forms g for its own edges, so one backward step is two launches (factors,
// variable sums). The potentials are clipped to +-1e6 before the loop (bp.py:85-87): a clipped
// entry gets no gradient.
//
// Checkpointing: the caller keeps the messages every k iterations (pgbp_run called k iterations
// at a time). Each chunk is recomputed here by a forward step with the engine's arithmetic (same
// operations in the same order, so the recomputed messages are the forward's), also storing
// every iteration's variable sums, then walked backwards. The recomputation of chunk c - 1 runs on
// a second stream while chunk c is walked backwards (two trajectory buffers), so the two chains
// of small launches overlap.
// Arrays here are in the caller's [B, n] layout; one thread per (unit, instance), consecutive
// threads on consecutive units of one instance.
#include <math.h>

#include <algorithm>
#include <mutex>

#include "pgbp_internal.h"

namespace pgbp {
namespace {

constexpr float kMsgNegInf = -1e32f;  // MSG_NEG_INF (pgmax/utils/__init__.py)
constexpr float kLpClip = 1e6f;       // potentials are clipped to +-1e6 (bp.py:85-87)

// NaN-propagating maximum (jnp.maximum): one max.NaN instruction.
__device__ __forceinline__ float maxn(float a, float b) {
  float r;
  asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}

// x / t; a power-of-two t multiplies by its exact reciprocal (the same correctly rounded value).
__device__ __forceinline__ float div_t(float x, float t) {
  const unsigned u = __float_as_uint(t);
  const unsigned e = (u >> 23) & 0xffu;
  if ((u & 0x807fffffu) == 0u && e >= 2u && e <= 252u) return x * __uint_as_float((254u - e) << 23);
  return x / t;
}

__device__ __forceinline__ float clip_lp(float x) { return fminf(fmaxf(x, -kLpClip), kLpClip); }

// The per-iteration kernels below (variable sums, forward and backward pairwise passes,
// gradient sums) begin with pdl_begin() and are launched with launch_pdl (pgbp_internal.h).

// vsum[b, v] = ev[b, v] + sum of m[b, e] over the edge states e of v, in increasing e (the
// reference's scatter order).
__global__ void __launch_bounds__(256) vsum_kernel(const int32_t* __restrict__ vs_off,
                                                   const int32_t* __restrict__ vs_edges,
                                                   int64_t nvs, const float* __restrict__ m,
                                                   int64_t n_es, const float* __restrict__ ev,
                                                   int64_t evs, float* __restrict__ vsum,
                                                   int64_t B) {
  pdl_begin();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nvs * B;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / nvs, v = i % nvs;
    float s = ev[b * evs + v];
    for (int32_t k = vs_off[v]; k < vs_off[v + 1]; ++k) s += m[b * n_es + vs_edges[k]];
    vsum[i] = s;
  }
}

// The forward quantities of one (dense pairwise factor, instance) with n1, n2 <= M: old messages
// o, variable-to-factor messages v, per-state maxima mx and sums of exponentials se, and the
// factor messages f, in the engine's operation order (pairwise_body, pgbp_kernels.cu).
template <int M>
struct Pair {
  float o1[M], o2[M], v1[M], v2[M], mx1[M], mx2[M], se1[M], se2[M], f1[M], f2[M];
};

template <int M>
__device__ __forceinline__ void pair_forward(Pair<M>& st, const int4 q, int n1, int n2,
                                             const float* __restrict__ m,
                                             const float* __restrict__ vsum,
                                             const float* __restrict__ lpb, float t) {
  constexpr int U = M <= 8 ? M : 1;
#pragma unroll U
  for (int a = 0; a < M; ++a)
    if (a < n1) {
      st.o1[a] = m[q.x + a];
      st.v1[a] = vsum[q.z + a] - st.o1[a];
      st.mx1[a] = -INFINITY;
      st.se1[a] = 0.0f;
    }
#pragma unroll U
  for (int c = 0; c < M; ++c)
    if (c < n2) {
      st.o2[c] = m[q.x + n1 + c];
      st.v2[c] = vsum[q.w + c] - st.o2[c];
      st.mx2[c] = -INFINITY;
      st.se2[c] = 0.0f;
    }
#pragma unroll U
  for (int a = 0; a < M; ++a)
#pragma unroll U
    for (int c = 0; c < M; ++c)
      if (a < n1 && c < n2) {
        const float s = ((0.0f + st.v1[a]) + st.v2[c]) + clip_lp(lpb[a * n2 + c]);
        st.mx1[a] = maxn(st.mx1[a], s);
        st.mx2[c] = maxn(st.mx2[c], s);
      }
#pragma unroll U
  for (int a = 0; a < M; ++a)
#pragma unroll U
    for (int c = 0; c < M; ++c)
      if (a < n1 && c < n2) {
        const float s = ((0.0f + st.v1[a]) + st.v2[c]) + clip_lp(lpb[a * n2 + c]);
        st.se1[a] += expf(div_t(s - st.mx1[a], t));
        st.se2[c] += expf(div_t(s - st.mx2[c], t));
      }
#pragma unroll U
  for (int a = 0; a < M; ++a)
    if (a < n1) st.f1[a] = (t * logf(st.se1[a]) + st.mx1[a]) - st.v1[a];
#pragma unroll U
  for (int c = 0; c < M; ++c)
    if (c < n2) st.f2[c] = (t * logf(st.se2[c]) + st.mx2[c]) - st.v2[c];
}

// Damping, normalisation and clipping of one edge with k <= M states (bp.py:127-133).
// M = 0: k bounds the loops at run time (edges of any size).
template <int M>
__device__ __forceinline__ void edge_forward(const float* o, const float* f, int k, float d,
                                             float omd, float* __restrict__ out) {
  constexpr int U = M > 0 && M <= 8 ? M : 1;
  const int n = M > 0 ? M : k;
  float mx = -INFINITY;
#pragma unroll U
  for (int s = 0; s < n; ++s)
    if (s < k) mx = maxn(mx, d * o[s] + omd * f[s]);
#pragma unroll U
  for (int s = 0; s < n; ++s)
    if (s < k) out[s] = maxn((d * o[s] + omd * f[s]) - mx, kMsgNegInf);
}

// Backward of edge_forward. g: dL/d(new messages) of the edge. Writes dL/df to gf and the damping
// path dL/do to gdir.
template <int M>
__device__ __forceinline__ void edge_backward(const float* o, const float* f, int k, float d,
                                              float omd, const float* g, float* gf,
                                              float* __restrict__ gdir) {
  constexpr int U = M > 0 && M <= 8 ? M : 1;
  const int n = M > 0 ? M : k;
  int arg = 0;
  float nmax = d * o[0] + omd * f[0];
#pragma unroll U
  for (int s = 1; s < n; ++s)
    if (s < k) {
      const float n = d * o[s] + omd * f[s];
      if (n > nmax) {
        nmax = n;
        arg = s;
      }
    }
  float gsum = 0.0f;
#pragma unroll U
  for (int s = 0; s < n; ++s)
    if (s < k) {
      const float gy = ((d * o[s] + omd * f[s]) - nmax >= kMsgNegInf) ? g[s] : 0.0f;
      gf[s] = gy;
      gsum += gy;
    }
#pragma unroll U
  for (int s = 0; s < n; ++s)
    if (s < k) {
      const float gn = gf[s] - (s == arg ? gsum : 0.0f);
      gf[s] = omd * gn;
      gdir[s] = d * gn;
    }
}

struct PairArgs {
  const int4* __restrict__ rec;          // (first edge state, -, first var state 1, of var 2)
  const int32_t* __restrict__ cfg_begin;
  int64_t count;
  int n1, n2;
  int64_t n_es, nvs, np_, B;
  const float* __restrict__ lp;
  int64_t lps;
  float d, omd, t;
};

// One forward iteration of every factor of a bucket: m (iteration input, [B, E_s]) and its
// variable sums -> next messages.
template <int M>
__global__ void __launch_bounds__(256) pairwise_forward_kernel(PairArgs a, const float* m,
                                                               const float* vsum, float* out) {
  pdl_begin();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.count * a.B;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / a.count, u = i % a.count;
    const int4 q = a.rec[u];
    Pair<M> st;
    pair_forward<M>(st, q, a.n1, a.n2, m + b * a.n_es, vsum + b * a.nvs,
                    a.lp + b * a.lps + a.cfg_begin[u], a.t);
    float* o = out + b * a.n_es + q.x;
    edge_forward<M>(st.o1, st.f1, a.n1, a.d, a.omd, o);
    edge_forward<M>(st.o2, st.f2, a.n2, a.d, a.omd, o + a.n1);
  }
}

// dL/d(messages of the iteration after this one): explicit (gexp, the caller's gradient, for the
// last iteration) or formed from the step after: gdir + gvsum[v(e)] - gvtof.
struct GradIn {
  const float* __restrict__ gexp;
  const float* __restrict__ gdir;
  const float* __restrict__ gvsum;
  const float* __restrict__ gvtof;
};

// One backward iteration of every factor of a bucket.
template <int M>
__global__ void __launch_bounds__(256) pairwise_backward_kernel(PairArgs a, const float* m,
                                                                const float* vsum, GradIn gin,
                                                                float* __restrict__ gdir,
                                                                float* __restrict__ gvtof,
                                                                float* __restrict__ glp) {
  pdl_begin();
  constexpr int U = M <= 8 ? M : 1;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.count * a.B;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / a.count, u = i % a.count;
    const int4 q = a.rec[u];
    const int64_t k0 = a.cfg_begin[u];
    const float* lpb = a.lp + b * a.lps + k0;
    Pair<M> st;
    pair_forward<M>(st, q, a.n1, a.n2, m + b * a.n_es, vsum + b * a.nvs, lpb, a.t);
    const int64_t e1 = b * a.n_es + q.x, e2 = e1 + a.n1;
    float g1[M], g2[M];
    if (gin.gexp) {
#pragma unroll U
      for (int s = 0; s < M; ++s)
        if (s < a.n1) g1[s] = gin.gexp[e1 + s];
#pragma unroll U
      for (int s = 0; s < M; ++s)
        if (s < a.n2) g2[s] = gin.gexp[e2 + s];
    } else {
      const float* gv = gin.gvsum + b * a.nvs;
#pragma unroll U
      for (int s = 0; s < M; ++s)
        if (s < a.n1) g1[s] = (gin.gdir[e1 + s] + gv[q.z + s]) - gin.gvtof[e1 + s];
#pragma unroll U
      for (int s = 0; s < M; ++s)
        if (s < a.n2) g2[s] = (gin.gdir[e2 + s] + gv[q.w + s]) - gin.gvtof[e2 + s];
    }
    float gf1[M], gf2[M];
    edge_backward<M>(st.o1, st.f1, a.n1, a.d, a.omd, g1, gf1, gdir + e1);
    edge_backward<M>(st.o2, st.f2, a.n2, a.d, a.omd, g2, gf2, gdir + e2);
    // g1 / g2 become the accumulators of dL/dvtof
#pragma unroll U
    for (int s = 0; s < M; ++s)
      if (s < a.n1) g1[s] = -gf1[s];
#pragma unroll U
    for (int s = 0; s < M; ++s)
      if (s < a.n2) g2[s] = -gf2[s];
    float* glpb = glp + b * a.np_ + k0;
#pragma unroll U
    for (int x = 0; x < M; ++x)
#pragma unroll U
      for (int y = 0; y < M; ++y)
        if (x < a.n1 && y < a.n2) {
          const float raw = lpb[x * a.n2 + y];
          const float s = ((0.0f + st.v1[x]) + st.v2[y]) + clip_lp(raw);
          const float p1 = expf(div_t(s - st.mx1[x], a.t)) / st.se1[x];
          const float p2 = expf(div_t(s - st.mx2[y], a.t)) / st.se2[y];
          const float gs = gf1[x] * p1 + gf2[y] * p2;
          g1[x] += gs;
          g2[y] += gs;
          if (raw >= -kLpClip && raw <= kLpClip) glpb[x * a.n2 + y] += gs;
        }
#pragma unroll U
    for (int s = 0; s < M; ++s)
      if (s < a.n1) gvtof[e1 + s] = g1[s];
#pragma unroll U
    for (int s = 0; s < M; ++s)
      if (s < a.n2) gvtof[e2 + s] = g2[s];
  }
}

// Generic EnumFactors (Plan::enum_generic): a thread per (factor, instance), the factor's edge
// states in per-thread arrays of MAXES entries.
struct GenArgs {
  const int32_t* __restrict__ es_begin;
  const int32_t* __restrict__ n_es;
  const int32_t* __restrict__ edge_off;
  const int32_t* __restrict__ edge_size;
  const int32_t* __restrict__ edge_vs;
  const int32_t* __restrict__ row_begin;
  const int32_t* __restrict__ n_cfg;
  const int32_t* __restrict__ n_vars;
  const int32_t* __restrict__ cfg_begin;
  const int32_t* __restrict__ row_les;
  int64_t count;
  int64_t n_es_all, nvs, np_, B;
  const float* __restrict__ lp;
  int64_t lps;
  float d, omd, t;
};

template <int MAXES>
struct Gen {
  float o[MAXES], v[MAXES], mx[MAXES], se[MAXES], f[MAXES];
};

// The factor's forward quantities for one instance (enum.py:451-475, the engine's operations in
// its order: config sums in variable order, then max and exp-sum in increasing config order).
template <int MAXES>
__device__ __forceinline__ void gen_forward(Gen<MAXES>& st, const GenArgs& a, int64_t u,
                                            const float* __restrict__ m,
                                            const float* __restrict__ vsum,
                                            const float* __restrict__ lpb) {
  const int64_t e0 = a.es_begin[u];
  const int n = a.n_es[u], nv = a.n_vars[u], ncfg = a.n_cfg[u];
  const int32_t* rows0 = a.row_les + a.row_begin[u];
  int pos = 0;
  for (int j = a.edge_off[u]; j < a.edge_off[u + 1]; ++j) {
    const int k = a.edge_size[j];
    const int64_t vs0 = a.edge_vs[j];
    for (int i = 0; i < k; ++i) {
      st.o[pos + i] = m[e0 + pos + i];
      st.v[pos + i] = vsum[vs0 + i] - st.o[pos + i];
    }
    pos += k;
  }
  for (int e = 0; e < n; ++e) {
    st.mx[e] = -INFINITY;
    st.se[e] = 0.0f;
  }
  for (int c = 0; c < ncfg; ++c) {
    const int32_t* rows = rows0 + (int64_t)c * nv;
    float sum = 0.0f;
    for (int i = 0; i < nv; ++i) sum += st.v[rows[i]];
    sum = sum + clip_lp(lpb[c]);
    for (int i = 0; i < nv; ++i) st.mx[rows[i]] = maxn(st.mx[rows[i]], sum);
  }
  for (int c = 0; c < ncfg; ++c) {
    const int32_t* rows = rows0 + (int64_t)c * nv;
    float sum = 0.0f;
    for (int i = 0; i < nv; ++i) sum += st.v[rows[i]];
    sum = sum + clip_lp(lpb[c]);
    for (int i = 0; i < nv; ++i) st.se[rows[i]] += expf(div_t(sum - st.mx[rows[i]], a.t));
  }
  for (int e = 0; e < n; ++e) st.f[e] = (a.t * logf(st.se[e]) + st.mx[e]) - st.v[e];
}

template <int MAXES>
__global__ void __launch_bounds__(256) generic_forward_kernel(GenArgs a, const float* m,
                                                              const float* vsum, float* out) {
  pdl_begin();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.count * a.B;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / a.count, u = i % a.count;
    Gen<MAXES> st;
    gen_forward<MAXES>(st, a, u, m + b * a.n_es_all, vsum + b * a.nvs,
                       a.lp + b * a.lps + a.cfg_begin[u]);
    float* o = out + b * a.n_es_all + a.es_begin[u];
    int pos = 0;
    for (int j = a.edge_off[u]; j < a.edge_off[u + 1]; ++j) {
      const int k = a.edge_size[j];
      edge_forward<0>(st.o + pos, st.f + pos, k, a.d, a.omd, o + pos);
      pos += k;
    }
  }
}

template <int MAXES>
__global__ void __launch_bounds__(256) generic_backward_kernel(GenArgs a, const float* m,
                                                               const float* vsum, GradIn gin,
                                                               float* __restrict__ gdir,
                                                               float* __restrict__ gvtof,
                                                               float* __restrict__ glp) {
  pdl_begin();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.count * a.B;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / a.count, u = i % a.count;
    const int64_t k0 = a.cfg_begin[u];
    const float* lpb = a.lp + b * a.lps + k0;
    Gen<MAXES> st;
    gen_forward<MAXES>(st, a, u, m + b * a.n_es_all, vsum + b * a.nvs, lpb);
    const int64_t e0 = b * a.n_es_all + a.es_begin[u];
    const int n = a.n_es[u], nv = a.n_vars[u], ncfg = a.n_cfg[u];
    // g = dL/d(new messages) of the factor's edge states; gf = dL/df
    float g[MAXES], gf[MAXES];
    int pos = 0;
    for (int j = a.edge_off[u]; j < a.edge_off[u + 1]; ++j) {
      const int k = a.edge_size[j];
      const int64_t vs0 = a.edge_vs[j];
      for (int s = 0; s < k; ++s) {
        const int64_t e = e0 + pos + s;
        g[pos + s] = gin.gexp ? gin.gexp[e]
                              : (gin.gdir[e] + gin.gvsum[b * a.nvs + vs0 + s]) - gin.gvtof[e];
      }
      edge_backward<0>(st.o + pos, st.f + pos, k, a.d, a.omd, g + pos, gf + pos, gdir + e0 + pos);
      pos += k;
    }
    // g becomes the accumulator of dL/dvtof
    for (int e = 0; e < n; ++e) g[e] = -gf[e];
    const int32_t* rows0 = a.row_les + a.row_begin[u];
    float* glpb = glp + b * a.np_ + k0;
    for (int c = 0; c < ncfg; ++c) {
      const int32_t* rows = rows0 + (int64_t)c * nv;
      const float raw = lpb[c];
      float sum = 0.0f;
      for (int x = 0; x < nv; ++x) sum += st.v[rows[x]];
      sum = sum + clip_lp(raw);
      float gs = 0.0f;
      for (int x = 0; x < nv; ++x) {
        const int e = rows[x];
        gs += gf[e] * (expf(div_t(sum - st.mx[e], a.t)) / st.se[e]);
      }
      for (int x = 0; x < nv; ++x) g[rows[x]] += gs;
      if (raw >= -kLpClip && raw <= kLpClip) glpb[c] += gs;
    }
    for (int e = 0; e < n; ++e) gvtof[e0 + e] = g[e];
  }
}

// ---- OR / AND factors (Plan::logical), a thread per (factor, instance)
constexpr double kLowT = 0.5;  // TEMPERATURE_STABILITY_THRE, pgmax/factor/logical.py:33

// update_utils.py:150-166, the engine's operations
__device__ __forceinline__ float lae_t(float a, float b, float t) {
  const float mx = maxn(a, b);
  float mn;
  asm("min.NaN.f32 %0, %1, %2;" : "=f"(mn) : "f"(a), "f"(b));
  return t * log1pf(expf(div_t(mn - mx, t))) + mx;
}
// update_utils.py:134-147 and 169-190 (both log1mexp branches evaluated, as jnp.where does)
__device__ __forceinline__ float lme_t(float a, float b, float t, float eps) {
  const float x = div_t(a - b, t);
  const float u = logf(-expm1f(-x));
  const float w = log1pf(-expf(-x));
  const float v = t * ((x <= 0.693147182464599609375f) ? u : w) + a;
  return (a >= b + eps) ? v : -INFINITY;
}
// Partial derivatives of lae_t (value l) and lme_t.
__device__ __forceinline__ void d_lae(float a, float b, float l, float t, float& da, float& db) {
  da = expf(div_t(a - l, t));
  db = expf(div_t(b - l, t));
}
__device__ __forceinline__ void d_lme(float a, float b, float t, float eps, float& da, float& db) {
  if (!(a >= b + eps)) {
    da = 0.0f;
    db = 0.0f;
    return;
  }
  const float e = expf(div_t(b - a, t));
  da = 1.0f / (1.0f - e);
  db = -e / (1.0f - e);
}

struct LogArgs {
  const int32_t* __restrict__ par_begin;
  const int4* __restrict__ par;    // (first edge state, -, first variable state)
  const int4* __restrict__ child;
  int64_t count;
  int rel;  // relevant state: 1 for OR, 0 for AND
  int64_t n_es, nvs, B;
  float d, omd, t;
};

// A binary edge's current messages and variable-to-factor messages (rel, other) in one instance.
struct Bin {
  float o[2];
  float vr, vo;
};

__device__ __forceinline__ Bin load_bin(const int4 r, int rel, const float* __restrict__ m,
                                        const float* __restrict__ vsum) {
  Bin x;
  x.o[0] = m[r.x];
  x.o[1] = m[r.x + 1];
  const float v0 = vsum[r.z] - x.o[0], v1 = vsum[r.z + 1] - x.o[1];
  x.vr = rel ? v1 : v0;
  x.vo = rel ? v0 : v1;
  return x;
}

// The factor-level quantities of logical_unit (pgbp_kernels.cu), in its order of operations.
struct LogFac {
  int64_t p0, p1, arg, arg2;
  float fs_oth, fs_x, max1, max2, c_rel, c_oth, ch_rel;
  Bin c;
  bool low, single;
};

__device__ __forceinline__ LogFac log_factor(const LogArgs& a, int64_t f, const float* m,
                                             const float* vsum) {
  LogFac q;
  q.p0 = a.par_begin[f];
  q.p1 = a.par_begin[f + 1];
  q.low = (double)a.t < kLowT;
  q.single = q.p1 - q.p0 == 1;
  q.fs_oth = 0.0f;
  q.fs_x = 0.0f;
  q.max1 = -INFINITY;
  for (int64_t i = q.p0; i < q.p1; ++i) {
    const Bin x = load_bin(a.par[i], a.rel, m, vsum);
    q.fs_oth += x.vo;
    q.max1 = maxn(q.max1, x.vr - x.vo);
    q.fs_x += lae_t(x.vr, x.vo, a.t);
  }
  q.arg = q.p1 - 1;
  q.max2 = -INFINITY;
  q.arg2 = -1;
  {
    int64_t last = -1;
    for (int64_t i = q.p0; i < q.p1; ++i) {
      const Bin x = load_bin(a.par[i], a.rel, m, vsum);
      if (x.vr - x.vo == q.max1) last = i;
    }
    if (last >= 0) q.arg = last;
    for (int64_t i = q.p0; i < q.p1; ++i) {
      const Bin x = load_bin(a.par[i], a.rel, m, vsum);
      const float w = i == q.arg ? -INFINITY : x.vr - x.vo;
      q.max2 = maxn(q.max2, w);
    }
    for (int64_t i = q.p0; i < q.p1; ++i) {  // the last parent attaining max2
      const Bin x = load_bin(a.par[i], a.rel, m, vsum);
      if (i != q.arg && x.vr - x.vo == q.max2) q.arg2 = i;
    }
  }
  q.c = load_bin(a.child[f], a.rel, m, vsum);
  q.c_rel = q.c.vr;
  q.c_oth = q.c.vo;
  q.ch_rel = lme_t(q.fs_x, q.fs_oth, a.t, 1e-4f);
  if (q.low) q.ch_rel = maxn(q.ch_rel, lae_t(q.fs_oth + q.max1, q.fs_oth + q.max2, a.t));
  return q;
}

// Parent i's outputs (p_rel, p_oth) of logical_unit at T > 0.
__device__ __forceinline__ void log_parent(const LogArgs& a, const LogFac& q, int64_t i,
                                           const Bin& x, float& p_rel, float& p_oth) {
  if (q.single) {
    p_rel = q.c_rel;
    p_oth = q.c_oth;
    return;
  }
  const float lse = lae_t(x.vr, x.vo, a.t);
  const float fs_lse_wo = q.fs_x - lse;
  const float fs_oth_wo = q.fs_oth - x.vo;
  p_rel = q.c_rel + fs_lse_wo;
  const float opt1 = q.c_oth + fs_oth_wo;
  const float opt2 = q.c_rel + fs_lse_wo;
  const float opt3 = q.c_rel + fs_oth_wo;
  p_oth = lme_t(lae_t(opt1, opt2, a.t), opt3, a.t, 1e-4f);
  if (q.low) {
    const float fsp = fs_oth_wo + (i == q.arg ? q.max2 : q.max1);
    p_oth = maxn(p_oth, lae_t(opt1, q.c_rel + fsp, a.t));
  }
}

__global__ void __launch_bounds__(256) logical_forward_kernel(LogArgs a, const float* m,
                                                              const float* vsum, float* out) {
  pdl_begin();
  for (int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < a.count * a.B;
       it += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = it / a.count, f = it % a.count;
    const float* mb = m + b * a.n_es;
    const float* vb = vsum + b * a.nvs;
    float* ob = out + b * a.n_es;
    const LogFac q = log_factor(a, f, mb, vb);
    for (int64_t i = q.p0; i < q.p1; ++i) {
      const int4 r = a.par[i];
      const Bin x = load_bin(r, a.rel, mb, vb);
      float p_rel, p_oth;
      log_parent(a, q, i, x, p_rel, p_oth);
      float fo[2];
      fo[a.rel] = p_rel - p_oth;
      fo[1 - a.rel] = 0.0f;
      edge_forward<2>(x.o, fo, 2, a.d, a.omd, ob + r.x);
    }
    float fo[2];
    fo[a.rel] = q.ch_rel - q.fs_oth;
    fo[1 - a.rel] = 0.0f;
    edge_forward<2>(q.c.o, fo, 2, a.d, a.omd, ob + a.child[f].x);
  }
}

// dL/d(factor outputs) of a binary edge from the gradient of its next messages: g = gexp, or
// gdir + gvsum[v] - gvtof of the step after; writes the damping path into gdir.
__device__ __forceinline__ void edge_grad(const LogArgs& a, const GradIn& gin, int64_t b,
                                          const int4 r, const Bin& x, const float* fo,
                                          float* __restrict__ gdir, float* gf) {
  const int64_t e = b * a.n_es + r.x;
  float g[2];
  for (int s = 0; s < 2; ++s)
    g[s] = gin.gexp ? gin.gexp[e + s]
                    : (gin.gdir[e + s] + gin.gvsum[b * a.nvs + r.z + s]) - gin.gvtof[e + s];
  edge_backward<2>(x.o, fo, 2, a.d, a.omd, g, gf, gdir + e);
}

// The part of parent i's backward that involves its own outputs: from dPR = g, dPO = -g to the
// factor-level and child gradients, and dA = dL/d(fs_x - lse_i), dO = dL/d(fs_oth - vo_i).
struct ParentGrad {
  float dA, dO, dcr, dco, dmax1, dmax2;
};

__device__ __forceinline__ ParentGrad parent_grad(const LogArgs& a, const LogFac& q, int64_t i,
                                                  const Bin& x, float g) {
  ParentGrad r{0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  if (q.single) {
    r.dcr = g;
    r.dco = -g;
    return r;
  }
  const float t = a.t;
  float dPO = -g;
  const float lse = lae_t(x.vr, x.vo, t);
  const float A = q.fs_x - lse, O = q.fs_oth - x.vo;
  const float o1 = q.c_oth + O, o2 = q.c_rel + A, o3 = q.c_rel + O;
  const float qv = lae_t(o1, o2, t);
  const float po = lme_t(qv, o3, t, 1e-4f);
  if (q.low) {
    const float M = i == q.arg ? q.max2 : q.max1;
    const float lbx = q.c_rel + O + M;
    const float lb = lae_t(o1, lbx, t);
    if (lb > po) {
      float s1, s2;
      d_lae(o1, lbx, lb, t, s1, s2);
      r.dco += dPO * s1;
      r.dO += dPO * s1;
      r.dcr += dPO * s2;
      r.dO += dPO * s2;
      if (i == q.arg) r.dmax2 += dPO * s2;
      else r.dmax1 += dPO * s2;
      dPO = 0.0f;
    }
  }
  if (dPO != 0.0f) {
    float pq, p3, s1, s2;
    d_lme(qv, o3, t, 1e-4f, pq, p3);
    const float dq = dPO * pq, do3 = dPO * p3;
    d_lae(o1, o2, qv, t, s1, s2);
    const float do1 = dq * s1, do2 = dq * s2;
    r.dco += do1;
    r.dO += do1;
    r.dcr += do2;
    r.dA += do2;
    r.dcr += do3;
    r.dO += do3;
  }
  r.dcr += g;  // p_rel = c_rel + A
  r.dA += g;
  return r;
}

__global__ void __launch_bounds__(256) logical_backward_kernel(LogArgs a, const float* m,
                                                               const float* vsum, GradIn gin,
                                                               float* __restrict__ gdir,
                                                               float* __restrict__ gvtof) {
  pdl_begin();
  const int rel = a.rel, oth = 1 - a.rel;
  for (int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < a.count * a.B;
       it += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = it / a.count, f = it % a.count;
    const float* mb = m + b * a.n_es;
    const float* vb = vsum + b * a.nvs;
    const LogFac q = log_factor(a, f, mb, vb);
    const float t = a.t;
    // the child's output rel = ch_rel - fs_oth
    float gc;
    {
      float fo[2], gf[2];
      fo[rel] = q.ch_rel - q.fs_oth;
      fo[oth] = 0.0f;
      edge_grad(a, gin, b, a.child[f], q.c, fo, gdir, gf);
      gc = gf[rel];
    }
    float dFX = 0.0f, dFO = -gc, dmax1 = 0.0f, dmax2 = 0.0f, dcr = 0.0f, dco = 0.0f;
    {
      float dCR = gc;
      const float crl = lme_t(q.fs_x, q.fs_oth, t, 1e-4f);
      if (q.low) {
        const float xa = q.fs_oth + q.max1, xb = q.fs_oth + q.max2;
        const float lbc = lae_t(xa, xb, t);
        if (lbc > crl) {
          float sa, sb;
          d_lae(xa, xb, lbc, t, sa, sb);
          dFO += dCR * (sa + sb);
          dmax1 += dCR * sa;
          dmax2 += dCR * sb;
          dCR = 0.0f;
        }
      }
      if (dCR != 0.0f) {
        float pa, pb;
        d_lme(q.fs_x, q.fs_oth, t, 1e-4f, pa, pb);
        dFX += dCR * pa;
        dFO += dCR * pb;
      }
    }
    // parents, first pass: the factor-level sums of their gradients
    for (int64_t i = q.p0; i < q.p1; ++i) {
      const int4 r = a.par[i];
      const Bin x = load_bin(r, rel, mb, vb);
      float p_rel, p_oth, fo[2], gf[2];
      log_parent(a, q, i, x, p_rel, p_oth);
      fo[rel] = p_rel - p_oth;
      fo[oth] = 0.0f;
      edge_grad(a, gin, b, r, x, fo, gdir, gf);
      const ParentGrad pg = parent_grad(a, q, i, x, gf[rel]);
      dcr += pg.dcr;
      dco += pg.dco;
      dmax1 += pg.dmax1;
      dmax2 += pg.dmax2;
      dFX += pg.dA;
      dFO += pg.dO;
    }
    // second pass: each parent's variable-to-factor gradients
    for (int64_t i = q.p0; i < q.p1; ++i) {
      const int4 r = a.par[i];
      const Bin x = load_bin(r, rel, mb, vb);
      float p_rel, p_oth, fo[2], gf[2];
      log_parent(a, q, i, x, p_rel, p_oth);
      fo[rel] = p_rel - p_oth;
      fo[oth] = 0.0f;
      edge_grad(a, gin, b, r, x, fo, gdir, gf);
      const ParentGrad pg = parent_grad(a, q, i, x, gf[rel]);
      const float dl = dFX - pg.dA;
      float dvo = dFO - pg.dO, dvr = 0.0f;
      float sr, so;
      d_lae(x.vr, x.vo, lae_t(x.vr, x.vo, t), t, sr, so);
      dvr += dl * sr;
      dvo += dl * so;
      if (i == q.arg) {
        dvr += dmax1;
        dvo -= dmax1;
      }
      if (i == q.arg2) {
        dvr += dmax2;
        dvo -= dmax2;
      }
      const int64_t e = b * a.n_es + r.x;
      gvtof[e + rel] = dvr;
      gvtof[e + oth] = dvo;
    }
    const int64_t ec = b * a.n_es + a.child[f].x;
    gvtof[ec + rel] = dcr;
    gvtof[ec + oth] = dco;
  }
}

// gvsum[v] = sum_{e in v} gvtof[e]; gev[v] += gvsum[v].
__global__ void __launch_bounds__(256) gvsum_kernel(const int32_t* __restrict__ vs_off,
                                                    const int32_t* __restrict__ vs_edges,
                                                    int64_t nvs, const float* __restrict__ gvtof,
                                                    int64_t n_es, float* __restrict__ gvsum,
                                                    float* __restrict__ gev, int64_t B) {
  pdl_begin();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nvs * B;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / nvs, v = i % nvs;
    float s = 0.0f;
    for (int32_t k = vs_off[v]; k < vs_off[v + 1]; ++k) s += gvtof[b * n_es + vs_edges[k]];
    gvsum[i] = s;
    gev[i] += s;
  }
}

// The initial normalisation of run_with_diffs (bp.py:88-92), per (edge, instance):
// out = max(x - max_edge(x), MSG_NEG_INF).
__global__ void __launch_bounds__(256) normalize_kernel(const int32_t* __restrict__ edge_start,
                                                        int64_t ne, const float* __restrict__ x,
                                                        float* __restrict__ out, int64_t n_es,
                                                        int64_t B) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ne * B;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / ne, e = i % ne;
    const int32_t lo = edge_start[e], hi = edge_start[e + 1];
    float mx = -INFINITY;
    for (int32_t s = lo; s < hi; ++s) mx = maxn(mx, x[b * n_es + s]);
    for (int32_t s = lo; s < hi; ++s) out[b * n_es + s] = maxn(x[b * n_es + s] - mx, kMsgNegInf);
  }
}

// Backward of normalize_kernel; the incoming gradient is formed from the first iteration's step
// (gdir + gvsum[v(e)] - gvtof).
__global__ void __launch_bounds__(256) normalize_backward_kernel(
    const int32_t* __restrict__ edge_start, const int32_t* __restrict__ vs_of_es, int64_t ne,
    const float* __restrict__ x, GradIn gin, float* __restrict__ gx, int64_t n_es, int64_t nvs,
    int64_t B) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ne * B;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / ne, e = i % ne;
    const int32_t lo = edge_start[e], hi = edge_start[e + 1];
    const float* xb = x + b * n_es;
    auto g = [&](int32_t s) {
      const int64_t j = b * n_es + s;
      return gin.gexp ? gin.gexp[j]
                      : (gin.gdir[j] + gin.gvsum[b * nvs + vs_of_es[s]]) - gin.gvtof[j];
    };
    float mx = xb[lo];
    int32_t arg = lo;
    for (int32_t s = lo + 1; s < hi; ++s)
      if (xb[s] > mx) {
        mx = xb[s];
        arg = s;
      }
    float gsum = 0.0f;
    for (int32_t s = lo; s < hi; ++s) gsum += (xb[s] - mx >= kMsgNegInf) ? g(s) : 0.0f;
    for (int32_t s = lo; s < hi; ++s) {
      const float gy = (xb[s] - mx >= kMsgNegInf) ? g(s) : 0.0f;
      gx[b * n_es + s] = gy - (s == arg ? gsum : 0.0f);
    }
  }
}

// out[j] = sum over b (in increasing b) of acc[b, j]: gradients of inputs shared by the batch.
__global__ void __launch_bounds__(256) sum_rows_kernel(const float* __restrict__ acc, int64_t n,
                                                       int64_t B, float* __restrict__ out) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n;
       j += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int64_t b = 0; b < B; ++b) s += acc[b * n + j];
    out[j] = s;
  }
}

__global__ void __launch_bounds__(256) beliefs_vjp_kernel(const int32_t* __restrict__ vs_of_es,
                                                          int64_t n_es,
                                                          const float* __restrict__ gb,
                                                          int64_t gbs, float* __restrict__ gm,
                                                          int64_t B) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_es * B;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = i / n_es, e = i % n_es;
    gm[i] = gb[b * gbs + vs_of_es[e]];
  }
}

dim3 grid_for(int64_t n, int sm) {
  const int64_t g = (n + 255) / 256;
  return dim3((unsigned)std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)sm * 16)));
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

size_t floats(int64_t n) { return align_up(sizeof(float) * (size_t)std::max<int64_t>(n, 1)); }

int bucket_m(const PairwiseBucket& q) {
  const int n = std::max(q.n1, q.n2);
  return n <= 2 ? 2 : n <= 4 ? 4 : n <= 8 ? 8 : 64;
}

PairArgs pair_args(const Plan& p, const PairwiseBucket& q, int64_t B, const float* lp,
                   int64_t lps, float d, float omd, float t) {
  return PairArgs{q.rec, q.cfg_begin, q.count, q.n1, q.n2, p.num_edge_states, p.num_var_states,
                  p.num_potentials, B, lp, lps, d, omd, t};
}

GenArgs gen_args(const Plan& p, int64_t B, const float* lp, int64_t lps, float d, float omd,
                 float t) {
  const EnumGeneric& g = p.enum_generic;
  return GenArgs{g.es_begin, g.n_es, g.edge_off, g.edge_size, g.edge_vs, g.row_begin, g.n_cfg,
                 g.n_vars, g.cfg_begin, g.row_les, g.count, p.num_edge_states, p.num_var_states,
                 p.num_potentials, B, lp, lps, d, omd, t};
}

// The generic factors' per-thread array size: the smallest of 8, 32, 128, 512 that holds the
// largest factor's edge states.
int gen_maxes(const Plan& p) {
  const int m = p.enum_generic.max_es;
  return m <= 8 ? 8 : m <= 32 ? 32 : m <= 128 ? 128 : 512;
}

void launch_generic_forward(const Plan& p, const GenArgs& a, cudaStream_t s, const float* m,
                            const float* vsum, float* out) {
  if (a.count == 0) return;
  const dim3 grid = grid_for(a.count * a.B, p.sm_count);
  switch (gen_maxes(p)) {
    case 8: launch_pdl(s, grid, dim3(256), generic_forward_kernel<8>, a, m, vsum, out); break;
    case 32: launch_pdl(s, grid, dim3(256), generic_forward_kernel<32>, a, m, vsum, out); break;
    case 128: launch_pdl(s, grid, dim3(256), generic_forward_kernel<128>, a, m, vsum, out); break;
    default: launch_pdl(s, grid, dim3(256), generic_forward_kernel<512>, a, m, vsum, out); break;
  }
}

void launch_generic_backward(const Plan& p, const GenArgs& a, cudaStream_t s, const float* m,
                             const float* vsum, const GradIn& gin, float* gdir, float* gvtof,
                             float* glp) {
  if (a.count == 0) return;
  const dim3 grid = grid_for(a.count * a.B, p.sm_count);
  switch (gen_maxes(p)) {
    case 8:
      launch_pdl(s, grid, dim3(256), generic_backward_kernel<8>, a, m, vsum, gin, gdir, gvtof, glp);
      break;
    case 32:
      launch_pdl(s, grid, dim3(256), generic_backward_kernel<32>, a, m, vsum, gin, gdir, gvtof, glp);
      break;
    case 128:
      launch_pdl(s, grid, dim3(256), generic_backward_kernel<128>, a, m, vsum, gin, gdir, gvtof,
                 glp);
      break;
    default:
      launch_pdl(s, grid, dim3(256), generic_backward_kernel<512>, a, m, vsum, gin, gdir, gvtof,
                 glp);
      break;
  }
}

LogArgs log_args(const Plan& p, int w, int64_t B, float d, float omd, float t) {
  const LogicalSet& g = p.logical[w];
  return LogArgs{g.par_begin, g.par, g.child, g.count, g.off > 0 ? 1 : 0, p.num_edge_states,
                 p.num_var_states, B, d, omd, t};
}

template <int M>
void launch_forward_m(const PairArgs& a, int sm, cudaStream_t s, const float* m, const float* vsum,
                      float* out) {
  launch_pdl(s, grid_for(a.count * a.B, sm), dim3(256), pairwise_forward_kernel<M>, a, m, vsum,
             out);
}

template <int M>
void launch_backward_m(const PairArgs& a, int sm, cudaStream_t s, const float* m,
                       const float* vsum, const GradIn& gin, float* gdir, float* gvtof,
                       float* glp) {
  launch_pdl(s, grid_for(a.count * a.B, sm), dim3(256), pairwise_backward_kernel<M>, a, m, vsum,
             gin, gdir, gvtof, glp);
}

// One chunk's trajectory: messages [len][B][E_s] (normalised) and variable sums [len][B][N_vs].
struct Traj {
  float* m;
  float* vs;
  size_t m_step, vs_step;  // floats between iterations
};

// Recomputes the chunk that starts at checkpoint ck.
void recompute(const Plan& p, cudaStream_t s, int64_t B, const float* lp, int64_t lps,
               const float* ev, int64_t evs, const float* ck, int64_t len, float d, float omd,
               float t, const Traj& tr) {
  ProfileScope prof(kProfAdjoint, s);
  const int64_t n_es = p.num_edge_states, nvs = p.num_var_states;
  normalize_kernel<<<grid_for(p.num_edges * B, p.sm_count), 256, 0, s>>>(p.edge_start, p.num_edges,
                                                                       ck, tr.m, n_es, B);
  for (int64_t j = 0; j < len; ++j) {
    const float* mj = tr.m + j * tr.m_step;
    float* vj = tr.vs + j * tr.vs_step;
    launch_pdl(s, grid_for(nvs * B, p.sm_count), dim3(256), vsum_kernel, p.vs_off, p.vs_edges, nvs,
               mj, n_es, ev, evs, vj, B);
    if (j + 1 == len) break;
    float* next = tr.m + (j + 1) * tr.m_step;
    for (const PairwiseBucket& q : p.pairwise) {
      const PairArgs a = pair_args(p, q, B, lp, lps, d, omd, t);
      switch (bucket_m(q)) {
        case 2: launch_forward_m<2>(a, p.sm_count, s, mj, vj, next); break;
        case 4: launch_forward_m<4>(a, p.sm_count, s, mj, vj, next); break;
        case 8: launch_forward_m<8>(a, p.sm_count, s, mj, vj, next); break;
        default: launch_forward_m<64>(a, p.sm_count, s, mj, vj, next); break;
      }
    }
    launch_generic_forward(p, gen_args(p, B, lp, lps, d, omd, t), s, mj, vj, next);
    for (int w = 0; w < 2; ++w) {
      if (p.logical[w].count == 0) continue;
      const LogArgs la = log_args(p, w, B, d, omd, t);
      launch_pdl(s, grid_for(la.count * B, p.sm_count), dim3(256), logical_forward_kernel, la, mj,
                 (const float*)vj, next);
    }
  }
}

struct GradSet {
  float* gdir;
  float* gvtof;
  float* gvsum;
};

// One iteration backwards: from the gradient of its output (gin) to gdir / gvtof / gvsum of its
// input, accumulating glp [B, P] and gev [B, N_vs].
void backward_step(const Plan& p, cudaStream_t s, int64_t B, const float* lp, int64_t lps,
                   const float* m, const float* vsum, const GradIn& gin, const GradSet& out,
                   float* glp, float* gev, float d, float omd, float t) {
  ProfileScope prof(kProfAdjoint, s);
  for (const PairwiseBucket& q : p.pairwise) {
    const PairArgs a = pair_args(p, q, B, lp, lps, d, omd, t);
    switch (bucket_m(q)) {
      case 2: launch_backward_m<2>(a, p.sm_count, s, m, vsum, gin, out.gdir, out.gvtof, glp); break;
      case 4: launch_backward_m<4>(a, p.sm_count, s, m, vsum, gin, out.gdir, out.gvtof, glp); break;
      case 8: launch_backward_m<8>(a, p.sm_count, s, m, vsum, gin, out.gdir, out.gvtof, glp); break;
      default:
        launch_backward_m<64>(a, p.sm_count, s, m, vsum, gin, out.gdir, out.gvtof, glp);
        break;
    }
  }
  launch_generic_backward(p, gen_args(p, B, lp, lps, d, omd, t), s, m, vsum, gin, out.gdir,
                          out.gvtof, glp);
  for (int w = 0; w < 2; ++w) {
    if (p.logical[w].count == 0) continue;
    const LogArgs la = log_args(p, w, B, d, omd, t);
    launch_pdl(s, grid_for(la.count * B, p.sm_count), dim3(256), logical_backward_kernel, la, m,
               vsum, gin, out.gdir, out.gvtof);
  }
  launch_pdl(s, grid_for(p.num_var_states * B, p.sm_count), dim3(256), gvsum_kernel, p.vs_off,
             p.vs_edges, p.num_var_states, out.gvtof, p.num_edge_states, out.gvsum, gev, B);
}

// A second stream per device for the recomputation, created on first use and kept.
constexpr int kMaxDevices = 64;
std::mutex g_aux_mu;
cudaStream_t g_aux[kMaxDevices] = {};

cudaError_t aux_stream(int device, cudaStream_t* out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_aux_mu);
  if (!g_aux[device]) {
    cudaError_t e = cudaStreamCreateWithFlags(&g_aux[device], cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
  }
  *out = g_aux[device];
  return cudaSuccess;
}

}  // namespace

const char* adjoint_unsupported(const Plan& p) {
  if (p.shared_potentials)
    return "the adjoint needs one potential table per factor; the plan shares tables";
  if (p.pool.count > 0)
    return "the adjoint covers EnumFactors, OR and AND factors; the graph has Pool factors";
  return "";
}

size_t vjp_workspace_bytes(const Plan& p, int64_t B, int64_t iters, int64_t checkpoint_every,
                           bool ev_shared, bool lp_shared) {
  const int64_t it = std::max<int64_t>(iters, 1);
  const int64_t k = std::max<int64_t>(1, std::min(checkpoint_every, it));
  const int64_t n_es = p.num_edge_states, nvs = p.num_var_states;
  size_t n = 0;
  n += 2 * (size_t)k * (floats(n_es * B) + floats(nvs * B));  // two trajectory buffers
  n += 2 * (2 * floats(n_es * B) + floats(nvs * B));          // two gradient sets
  if (lp_shared) n += floats(p.num_potentials * B);
  if (ev_shared) n += floats(nvs * B);
  return n;
}

cudaError_t run_vjp(const Plan& p, cudaStream_t s, int64_t B, const float* lp, int64_t lp_stride,
                    const float* ev, int64_t ev_stride, const float* checkpoints, int64_t iters_in,
                    int64_t checkpoint_every, double damping, double temperature,
                    const float* g_msgs, float* g_lp, float* g_ev, float* g_msgs_in, void* ws,
                    size_t ws_bytes) {
  (void)ws_bytes;
  const int64_t iters = std::max<int64_t>(iters_in, 1);
  const int64_t k = std::max<int64_t>(1, std::min(checkpoint_every, iters));
  const int64_t n_ck = (iters + k - 1) / k;
  const int64_t n_es = p.num_edge_states, nvs = p.num_var_states, np_ = p.num_potentials;
  const bool lp_shared = lp_stride == 0, ev_shared = ev_stride == 0;
  char* w = static_cast<char*>(ws);
  auto take = [&](size_t bytes) {
    char* r = w;
    w += bytes;
    return reinterpret_cast<float*>(r);
  };
  Traj tr[2];
  for (Traj& x : tr) {
    x.m_step = floats(n_es * B) / sizeof(float);
    x.vs_step = floats(nvs * B) / sizeof(float);
    x.m = take((size_t)k * floats(n_es * B));
    x.vs = take((size_t)k * floats(nvs * B));
  }
  GradSet gs[2];
  for (GradSet& x : gs) {
    x.gdir = take(floats(n_es * B));
    x.gvtof = take(floats(n_es * B));
    x.gvsum = take(floats(nvs * B));
  }
  float* glp = lp_shared ? take(floats(np_ * B)) : g_lp;
  float* gev = ev_shared ? take(floats(nvs * B)) : g_ev;
  const float d = (float)damping, omd = (float)(1.0 - damping), t = (float)temperature;
  const size_t ck_step = (size_t)B * (size_t)n_es;
  auto chunk_len = [&](int64_t c) { return std::min(k, iters - c * k); };

  cudaStream_t aux = nullptr;
  cudaError_t e = aux_stream(p.device, &aux);
  if (e != cudaSuccess) return e;
  cudaEvent_t fork = nullptr, ev_r[2] = {nullptr, nullptr}, ev_b[2] = {nullptr, nullptr};
  auto cleanup = [&]() {
    for (cudaEvent_t x : {fork, ev_r[0], ev_r[1], ev_b[0], ev_b[1]})
      if (x) cudaEventDestroy(x);
  };
  for (cudaEvent_t* x : {&fork, &ev_r[0], &ev_r[1], &ev_b[0], &ev_b[1]}) {
    if ((e = cudaEventCreateWithFlags(x, cudaEventDisableTiming)) != cudaSuccess) {
      cleanup();
      return e;
    }
  }
  e = cudaMemsetAsync(glp, 0, sizeof(float) * (size_t)(np_ * B), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(gev, 0, sizeof(float) * (size_t)(nvs * B), s);
  // the recomputation reads what the caller wrote on its stream
  if (e == cudaSuccess) e = cudaEventRecord(fork, s);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(aux, fork, 0);
  if (e != cudaSuccess) {
    cleanup();
    return e;
  }
  recompute(p, aux, B, lp, lp_stride, ev, ev_stride, checkpoints + (n_ck - 1) * ck_step,
            chunk_len(n_ck - 1), d, omd, t, tr[(n_ck - 1) & 1]);
  cudaEventRecord(ev_r[(n_ck - 1) & 1], aux);
  GradIn gin{g_msgs, nullptr, nullptr, nullptr};
  int cur = 0;
  for (int64_t c = n_ck - 1; c >= 0; --c) {
    if (c >= 1) {
      // chunk c - 1 reuses the buffer of chunk c + 1: wait until that chunk has been walked
      if (c + 1 < n_ck) cudaStreamWaitEvent(aux, ev_b[(c + 1) & 1], 0);
      recompute(p, aux, B, lp, lp_stride, ev, ev_stride, checkpoints + (c - 1) * ck_step,
                chunk_len(c - 1), d, omd, t, tr[(c - 1) & 1]);
      cudaEventRecord(ev_r[(c - 1) & 1], aux);
    }
    cudaStreamWaitEvent(s, ev_r[c & 1], 0);
    const Traj& x = tr[c & 1];
    for (int64_t j = chunk_len(c) - 1; j >= 0; --j) {
      backward_step(p, s, B, lp, lp_stride, x.m + j * x.m_step, x.vs + j * x.vs_step, gin, gs[cur],
                    glp, gev, d, omd, t);
      gin = GradIn{nullptr, gs[cur].gdir, gs[cur].gvsum, gs[cur].gvtof};
      cur ^= 1;
    }
    cudaEventRecord(ev_b[c & 1], s);
  }
  {
    ProfileScope prof(kProfAdjoint, s);
    if (g_msgs_in)
      normalize_backward_kernel<<<grid_for(p.num_edges * B, p.sm_count), 256, 0, s>>>(
          p.edge_start, p.vs_of_es, p.num_edges, checkpoints, gin, g_msgs_in, n_es, nvs, B);
    if (lp_shared && np_ > 0)
      sum_rows_kernel<<<grid_for(np_, p.sm_count), 256, 0, s>>>(glp, np_, B, g_lp);
    if (ev_shared && nvs > 0)
      sum_rows_kernel<<<grid_for(nvs, p.sm_count), 256, 0, s>>>(gev, nvs, B, g_ev);
  }
  e = cudaGetLastError();
  cleanup();
  return e;
}

cudaError_t beliefs_vjp(const Plan& p, cudaStream_t s, int64_t B, const float* g_beliefs,
                        int64_t gb_stride, float* g_msgs) {
  ProfileScope prof(kProfReadout, s);
  beliefs_vjp_kernel<<<grid_for(p.num_edge_states * B, p.sm_count), 256, 0, s>>>(
      p.vs_of_es, p.num_edge_states, g_beliefs, gb_stride, g_msgs, B);
  return cudaGetLastError();
}

}  // namespace pgbp
