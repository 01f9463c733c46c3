// Energy of MAP decodings on the device: compute_energy (pgmax/infer/energy.py:53-148, without
// debug mode) with the per-type terms EnumFactor.compute_energy (pgmax/factor/enum.py:276-323),
// LogicalFactor.compute_energy (pgmax/factor/logical.py:295-358) and PoolFactor.compute_energy
// (pgmax/factor/pool.py:184-239). For instance b, with onehot_b(vs) = 1 when the decoded state of
// vs's variable is vs:
//
//   energy[b] = -sum_vs onehot_b(vs) * evidence[b, vs]            (every state: 0 * inf is nan)
//             + [Enum factors]  #decoded configs != #factors ? +inf : -sum lp[b, decoded configs]
//             + [OR factors]    (all parents in state 0) != (child in state 0) for some factor ? +inf : 0
//             + [AND factors]   the same with state 1
//             + [Pool factors]  #choices in state 1 != (indicator in state 1) for some factor ? +inf : 0
//
// A term is added only when the graph has factors of its type (energy.py:140-147). A config of an
// Enum factor is decoded when every one of its variables is in the config's state; the dense
// pairwise factors list every config, so one config is decoded unless a state is out of range.
// The decoded state of a variable with K states is map[b, v], a negative state taken as
// map[b, v] + K (the reference indexes its one-hot with it, and JAX wraps a negative index once);
// outside [0, K) no state of the variable is decoded, as JAX drops out-of-range scatters.
//
// Work: items are variables (the evidence term) and factors of each kind, in segments; a CTA takes
// kEnergyChunk items of one segment for one instance and reduces them in double, in a fixed order,
// into one partial; a second kernel (a warp per instance) adds the partials in a fixed order. The
// result does not depend on timing. Loads per instance: the decoded states, the evidence, one
// potential per decoded Enum config and the plan's index arrays (shared by the batch, L2-resident).

#include <math.h>

#include <algorithm>

#include "pgbp_internal.h"

namespace pgbp {
namespace {

constexpr int kEnergyThreads = 256;
constexpr int kEnergyChunk = 4 * kEnergyThreads;
constexpr int kMaxSegsPerLaunch = 32;

enum : int { kFlagOr = 1, kFlagAnd = 2, kFlagPool = 4 };

struct EnergyPartial {
  double u;        // sum of onehot * evidence
  double e;        // sum of the decoded configs' potentials
  long long cnt;   // decoded Enum configs
  int flags;       // violated OR / AND / Pool constraints
  int pad;
};
static_assert(sizeof(EnergyPartial) == 32, "partial layout");

// One segment as the kernel sees it: pointers of its factor kind. a = n1 (pairwise) or the
// relevant state (logical); b = n2 (pairwise).
struct SegDev {
  int kind, a, b, pad;
  int64_t items, chunk_begin;
  const void* p0;
  const void* p1;
  const void* p2;
  const int32_t* fac;  // item -> factor index in the flat wiring (factor segments)
};

struct Launch {
  int nseg;
  SegDev seg[kMaxSegsPerLaunch];
};

struct Args {
  const int32_t* var_off;
  const int32_t* var_of_vs;
  const float* lp;
  int64_t lps;
  const float* ev;
  int64_t evs;
  const int32_t* map;
  int64_t ms;
  int64_t B;
  int64_t chunks;
  EnumGeneric gen;
};

// Decoded state of variable v, or -1 when no state is decoded.
__device__ __forceinline__ int decoded_state(const int32_t* __restrict__ map_b,
                                             const int32_t* __restrict__ var_off, int v) {
  const int k = __ldg(var_off + v + 1) - __ldg(var_off + v);
  int s = map_b[v];
  if (s < 0) s += k;
  return (s >= 0 && s < k) ? s : -1;
}

__device__ __forceinline__ int state_of_vs(const int32_t* __restrict__ map_b, const Args& a,
                                           int vs0) {
  return decoded_state(map_b, a.var_off, __ldg(a.var_of_vs + vs0));
}

__device__ __forceinline__ void energy_item(const Args& a, const SegDev& sg, int64_t i,
                                            const int32_t* __restrict__ map_b,
                                            const float* __restrict__ ev_b,
                                            const float* __restrict__ lp_b, double& u, double& e,
                                            long long& cnt, int& flags) {
  switch (sg.kind) {
    case kEnergyVars: {
      const int v = (int)i;
      const int vs0 = __ldg(a.var_off + v), k = __ldg(a.var_off + v + 1) - vs0;
      const int s = decoded_state(map_b, a.var_off, v);
      for (int t = 0; t < k; ++t) u += (t == s ? 1.0 : 0.0) * (double)ev_b[vs0 + t];
      break;
    }
    case kEnergyPairwise: {
      const int4 r = __ldg(static_cast<const int4*>(sg.p0) + i);
      const int sa = state_of_vs(map_b, a, r.z), sb = state_of_vs(map_b, a, r.w);
      if (sa >= 0 && sb >= 0) {
        ++cnt;
        e += (double)lp_b[__ldg(static_cast<const int32_t*>(sg.p1) + i) + sa * sg.b + sb];
      }
      break;
    }
    case kEnergyGeneric: {
      const EnumGeneric& g = a.gen;
      const int j0 = __ldg(g.edge_off + i), nv = __ldg(g.n_vars + i), nc = __ldg(g.n_cfg + i);
      const int rb = __ldg(g.row_begin + i), cb = __ldg(g.cfg_begin + i);
      bool any = true;
      for (int t = 0; t < nv && any; ++t) any = state_of_vs(map_b, a, __ldg(g.edge_vs + j0 + t)) >= 0;
      if (!any) break;  // a variable decodes no state: no config of the factor is decoded
      for (int c = 0; c < nc; ++c) {
        int est = 0;
        bool ok = true;
        for (int t = 0; t < nv; ++t) {
          const int j = j0 + t;
          const int s = state_of_vs(map_b, a, __ldg(g.edge_vs + j));
          if (__ldg(g.row_les + rb + c * nv + t) != est + s) {
            ok = false;
            break;
          }
          est += __ldg(g.edge_size + j);
        }
        if (ok) {
          ++cnt;
          e += (double)lp_b[cb + c];
        }
      }
      break;
    }
    case kEnergyLogical: {
      const int32_t* pb = static_cast<const int32_t*>(sg.p0);
      const int4* par = static_cast<const int4*>(sg.p1);
      const int4* ch = static_cast<const int4*>(sg.p2);
      const int r = sg.a;
      bool all = true;
      for (int q = __ldg(pb + i), q1 = __ldg(pb + i + 1); q < q1 && all; ++q)
        all = state_of_vs(map_b, a, __ldg(par + q).z) == r;
      const bool child = state_of_vs(map_b, a, __ldg(ch + i).z) == r;
      if (all != child) flags |= r == 0 ? kFlagOr : kFlagAnd;
      break;
    }
    case kEnergyPool: {
      const int32_t* cbg = static_cast<const int32_t*>(sg.p0);
      const int4* chs = static_cast<const int4*>(sg.p1);
      const int4* ind = static_cast<const int4*>(sg.p2);
      int on = 0;
      for (int q = __ldg(cbg + i), q1 = __ldg(cbg + i + 1); q < q1; ++q)
        on += state_of_vs(map_b, a, __ldg(chs + q).z) == 1;
      const int ind_on = state_of_vs(map_b, a, __ldg(ind + i).z) == 1;
      if (on != ind_on) flags |= kFlagPool;
      break;
    }
    default:
      break;
  }
}

__device__ __forceinline__ void warp_reduce(double& u, double& e, long long& cnt, int& flags) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    u += __shfl_xor_sync(0xffffffffu, u, o);
    e += __shfl_xor_sync(0xffffffffu, e, o);
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    flags |= __shfl_xor_sync(0xffffffffu, flags, o);
  }
}

// Decoded states with the instances innermost: map_t[v * B + b] = map[b * ms + v] (the bits as
// given), 32 x 32 tiles through shared memory.
__global__ void transpose_states_kernel(const int32_t* __restrict__ map, int64_t ms, int64_t nv,
                                        int64_t B, int32_t* __restrict__ map_t) {
  __shared__ int32_t tile[32][33];
  const int64_t v0 = (int64_t)blockIdx.x * 32, b0 = (int64_t)blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t b = b0 + r, v = v0 + threadIdx.x;
    if (b < B && v < nv) tile[r][threadIdx.x] = map[b * ms + v];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t v = v0 + r, b = b0 + threadIdx.x;
    if (v < nv && b < B) map_t[v * B + b] = tile[threadIdx.x][r];
  }
}

// Dense pairwise segments with the instances on the lanes: grid (chunks of the segment,
// ceil(B / 32)). Warp w of a CTA takes factors w, w + 8, ... of the chunk for 32 instances, so a
// factor's record, variables and state counts are loaded once per 32 instances and the decoded
// states are read as coalesced rows of map_t; each lane sums its instance in double in factor
// order and the eight warps are added in warp order (a fixed order: the result does not depend
// on timing).
__global__ void __launch_bounds__(kEnergyThreads) energy_pairwise_kernel(
    Args a, SegDev sg, const int32_t* __restrict__ map_t, EnergyPartial* part) {
  __shared__ double s_e[kEnergyThreads / 32][32];
  __shared__ long long s_c[kEnergyThreads / 32][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t chunk = sg.chunk_begin + blockIdx.x;
  const int64_t i0 = (int64_t)blockIdx.x * kEnergyChunk;
  const int64_t i1 = i0 + kEnergyChunk < sg.items ? i0 + kEnergyChunk : sg.items;
  const int64_t b = (int64_t)blockIdx.y * 32 + lane;
  const bool valid = b < a.B;
  const float* __restrict__ lp_b = a.lp + (valid ? b : 0) * a.lps;
  const int4* __restrict__ rec = static_cast<const int4*>(sg.p0);
  const int32_t* __restrict__ cfg = static_cast<const int32_t*>(sg.p1);
  // a bucket's factors all have n1 and n2 states (sg.a, sg.b); four factors per step, their
  // loads issued level by level (record, variables, decoded states, potential) so the four
  // dependent chains overlap; the sums still run in factor order
  constexpr int kStep = 4, kWarps = kEnergyThreads / 32;
  const int ka = sg.a, kb = sg.b;
  double e = 0.0;
  long long cnt = 0;
  for (int64_t i = i0 + warp; i < i1; i += kStep * kWarps) {
    int4 r[kStep];
    int k0[kStep], va[kStep], vb[kStep], sa[kStep], sb[kStep];
    bool in[kStep];
    float pv[kStep];
#pragma unroll
    for (int u = 0; u < kStep; ++u) {
      const int64_t f = i + (int64_t)u * kWarps;
      in[u] = f < i1;
      r[u] = in[u] ? __ldg(rec + f) : make_int4(0, 0, 0, 0);
      k0[u] = in[u] ? __ldg(cfg + f) : 0;
    }
#pragma unroll
    for (int u = 0; u < kStep; ++u) {
      va[u] = in[u] ? __ldg(a.var_of_vs + r[u].z) : 0;
      vb[u] = in[u] ? __ldg(a.var_of_vs + r[u].w) : 0;
    }
#pragma unroll
    for (int u = 0; u < kStep; ++u) {
      sa[u] = (valid && in[u]) ? map_t[(int64_t)va[u] * a.B + b] : -1 - ka;
      sb[u] = (valid && in[u]) ? map_t[(int64_t)vb[u] * a.B + b] : -1 - kb;
      if (sa[u] < 0) sa[u] += ka;
      if (sb[u] < 0) sb[u] += kb;
      in[u] = sa[u] >= 0 && sa[u] < ka && sb[u] >= 0 && sb[u] < kb;
      pv[u] = in[u] ? lp_b[k0[u] + sa[u] * kb + sb[u]] : 0.0f;
    }
#pragma unroll
    for (int u = 0; u < kStep; ++u) {
      if (in[u]) {
        ++cnt;
        e += (double)pv[u];
      }
    }
  }
  s_e[warp][lane] = e;
  s_c[warp][lane] = cnt;
  __syncthreads();
  if (warp == 0 && valid) {
    for (int w = 1; w < kEnergyThreads / 32; ++w) {
      e += s_e[w][lane];
      cnt += s_c[w][lane];
    }
    EnergyPartial q;
    q.u = 0.0;
    q.e = e;
    q.cnt = cnt;
    q.flags = 0;
    q.pad = 0;
    part[b * a.chunks + chunk] = q;
  }
}

// grid (chunks of this launch, min(B, 65535)); partials [B][a.chunks]. With skip_pairwise the
// dense pairwise chunks are left to energy_pairwise_kernel.
__global__ void __launch_bounds__(kEnergyThreads) energy_partial_kernel(Args a, Launch L,
                                                                         int64_t first_chunk,
                                                                         int skip_pairwise,
                                                                         EnergyPartial* part) {
  __shared__ double s_u[kEnergyThreads / 32], s_e[kEnergyThreads / 32];
  __shared__ long long s_c[kEnergyThreads / 32];
  __shared__ int s_f[kEnergyThreads / 32];
  const int64_t chunk = first_chunk + blockIdx.x;
  int si = 0;
  while (si + 1 < L.nseg && L.seg[si + 1].chunk_begin <= chunk) ++si;
  const SegDev sg = L.seg[si];
  if (skip_pairwise && sg.kind == kEnergyPairwise) return;
  const int64_t i0 = (chunk - sg.chunk_begin) * kEnergyChunk;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t b = blockIdx.y; b < a.B; b += gridDim.y) {
    const int32_t* map_b = a.map + b * a.ms;
    const float* ev_b = a.ev ? a.ev + b * a.evs : nullptr;
    const float* lp_b = a.lp ? a.lp + b * a.lps : nullptr;
    double u = 0.0, e = 0.0;
    long long cnt = 0;
    int flags = 0;
    for (int k = 0; k < kEnergyChunk / kEnergyThreads; ++k) {
      const int64_t i = i0 + (int64_t)k * kEnergyThreads + threadIdx.x;
      if (i < sg.items) energy_item(a, sg, i, map_b, ev_b, lp_b, u, e, cnt, flags);
    }
    warp_reduce(u, e, cnt, flags);
    if (lane == 0) {
      s_u[warp] = u;
      s_e[warp] = e;
      s_c[warp] = cnt;
      s_f[warp] = flags;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int w = 1; w < kEnergyThreads / 32; ++w) {
        u += s_u[w];
        e += s_e[w];
        cnt += s_c[w];
        flags |= s_f[w];
      }
      EnergyPartial r;
      r.u = u;
      r.e = e;
      r.cnt = cnt;
      r.flags = flags;
      r.pad = 0;
      part[b * a.chunks + chunk] = r;
    }
    __syncthreads();
  }
}

// compute_energy's debug mode (pgmax/infer/energy.py:151-204) for B decodings: per variable
// -evidence[state] (NaN when no state is decoded); per factor the decoded config, which the host
// turns into the factor's energy with the factor's own potentials: an EnumFactor's index of the
// decoded config among its configs, the last of equal configs as the reference's lookup keeps it
// (-1 when none is decoded, enum.py:326-360); 0 / -1 for an OR / AND (logical.py:378-406) or Pool
// (pool.py:242-272) factor that the decoding satisfies / violates. grid (chunks of this launch,
// min(B, 65535)); var_e [B][num_variables], fac_cfg [B][num_factors].
__global__ void __launch_bounds__(kEnergyThreads) energy_terms_kernel(Args a, Launch L,
                                                                       int64_t first_chunk,
                                                                       int64_t nv, int64_t nf,
                                                                       float* __restrict__ var_e,
                                                                       int32_t* __restrict__ fac_cfg) {
  const int64_t chunk = first_chunk + blockIdx.x;
  int si = 0;
  while (si + 1 < L.nseg && L.seg[si + 1].chunk_begin <= chunk) ++si;
  const SegDev sg = L.seg[si];
  const int64_t i0 = (chunk - sg.chunk_begin) * kEnergyChunk;
  for (int64_t b = blockIdx.y; b < a.B; b += gridDim.y) {
    const int32_t* map_b = a.map + b * a.ms;
    const float* ev_b = a.ev ? a.ev + b * a.evs : nullptr;
    for (int k = 0; k < kEnergyChunk / kEnergyThreads; ++k) {
      const int64_t i = i0 + (int64_t)k * kEnergyThreads + threadIdx.x;
      if (i >= sg.items) continue;
      int cfg = -1;
      switch (sg.kind) {
        case kEnergyVars: {
          const int v = (int)i;
          const int s = decoded_state(map_b, a.var_off, v);
          var_e[b * nv + v] = s >= 0 ? -ev_b[__ldg(a.var_off + v) + s] : NAN;
          continue;
        }
        case kEnergyPairwise: {
          const int4 r = __ldg(static_cast<const int4*>(sg.p0) + i);
          const int sa = state_of_vs(map_b, a, r.z), sb = state_of_vs(map_b, a, r.w);
          if (sa >= 0 && sb >= 0) cfg = sa * sg.b + sb;   // row-major configs
          break;
        }
        case kEnergyGeneric: {
          const EnumGeneric& g = a.gen;
          const int j0 = __ldg(g.edge_off + i), nvf = __ldg(g.n_vars + i), nc = __ldg(g.n_cfg + i);
          const int rb = __ldg(g.row_begin + i);
          for (int c = 0; c < nc; ++c) {
            int est = 0;
            bool ok = true;
            for (int t = 0; t < nvf && ok; ++t) {
              const int j = j0 + t;
              const int s = state_of_vs(map_b, a, __ldg(g.edge_vs + j));
              ok = s >= 0 && __ldg(g.row_les + rb + c * nvf + t) == est + s;
              est += __ldg(g.edge_size + j);
            }
            if (ok) cfg = c;
          }
          break;
        }
        case kEnergyLogical: {
          const int32_t* pb = static_cast<const int32_t*>(sg.p0);
          const int4* par = static_cast<const int4*>(sg.p1);
          const int4* ch = static_cast<const int4*>(sg.p2);
          const int r = sg.a;
          bool all = true;
          for (int q = __ldg(pb + i), q1 = __ldg(pb + i + 1); q < q1 && all; ++q)
            all = state_of_vs(map_b, a, __ldg(par + q).z) == r;
          const bool child = state_of_vs(map_b, a, __ldg(ch + i).z) == r;
          cfg = all != child ? -1 : 0;
          break;
        }
        case kEnergyPool: {
          const int32_t* cbg = static_cast<const int32_t*>(sg.p0);
          const int4* chs = static_cast<const int4*>(sg.p1);
          const int4* ind = static_cast<const int4*>(sg.p2);
          int on = 0;
          for (int q = __ldg(cbg + i), q1 = __ldg(cbg + i + 1); q < q1; ++q)
            on += state_of_vs(map_b, a, __ldg(chs + q).z) == 1;
          const int ind_on = state_of_vs(map_b, a, __ldg(ind + i).z) == 1;
          cfg = on != ind_on ? -1 : 0;
          break;
        }
        default:
          continue;
      }
      fac_cfg[b * nf + __ldg(sg.fac + i)] = cfg;
    }
  }
}

// One warp per instance: adds its partials (lane c, c + 32, ... then a fixed butterfly) and
// combines the terms in the reference's order.
__global__ void energy_final_kernel(const EnergyPartial* __restrict__ part, int64_t chunks,
                                    int64_t B, long long num_enum, int present, float* out) {
  const int lane = threadIdx.x & 31;
  const int64_t b = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (b >= B) return;
  double u = 0.0, e = 0.0;
  long long cnt = 0;
  int flags = 0;
  for (int64_t c = lane; c < chunks; c += 32) {
    const EnergyPartial r = part[b * chunks + c];
    u += r.u;
    e += r.e;
    cnt += r.cnt;
    flags |= r.flags;
  }
  warp_reduce(u, e, cnt, flags);
  if (lane != 0) return;
  double en = -u;
  if (present & 1) en += cnt != num_enum ? (double)INFINITY : -e;
  if (present & 2) en += (flags & kFlagOr) ? (double)INFINITY : 0.0;
  if (present & 4) en += (flags & kFlagAnd) ? (double)INFINITY : 0.0;
  if (present & 8) en += (flags & kFlagPool) ? (double)INFINITY : 0.0;
  out[b] = (float)en;
}

int64_t chunks_of(int64_t items) { return (items + kEnergyChunk - 1) / kEnergyChunk; }

// A segment's pointers as the kernels see them.
SegDev seg_dev(const Plan& p, const EnergySeg& es) {
  SegDev d{};
  d.kind = es.kind;
  d.items = es.items;
  d.chunk_begin = es.chunk_begin;
  switch (es.kind) {
    case kEnergyPairwise: {
      const PairwiseBucket& q = p.pairwise[(size_t)es.param];
      d.a = q.n1;
      d.b = q.n2;
      d.p0 = q.rec;
      d.p1 = q.cfg_begin;
      d.fac = q.fac;
      break;
    }
    case kEnergyGeneric:
      d.fac = p.enum_generic.fac;
      break;
    case kEnergyLogical: {
      const LogicalSet& g = p.logical[es.param];
      d.a = g.off == 1 ? 0 : 1;  // the relevant state: 0 for OR, 1 for AND
      d.p0 = g.par_begin;
      d.p1 = g.par;
      d.p2 = g.child;
      d.fac = g.fac;
      break;
    }
    case kEnergyPool:
      d.p0 = p.pool.ch_begin;
      d.p1 = p.pool.ch;
      d.p2 = p.pool.ind;
      d.fac = p.pool.fac;
      break;
    default:
      break;
  }
  return d;
}

}  // namespace

void energy_plan(Plan& p) {
  p.energy_segs.clear();
  int64_t c = 0;
  auto add = [&](int kind, int param, int64_t items) {
    if (items <= 0) return;
    EnergySeg s;
    s.kind = kind;
    s.param = param;
    s.items = items;
    s.chunk_begin = c;
    c += chunks_of(items);
    p.energy_segs.push_back(s);
  };
  add(kEnergyVars, 0, p.num_variables);
  for (size_t q = 0; q < p.pairwise.size(); ++q) add(kEnergyPairwise, (int)q, p.pairwise[q].count);
  add(kEnergyGeneric, 0, p.enum_generic.count);
  add(kEnergyLogical, 0, p.logical[0].count);
  add(kEnergyLogical, 1, p.logical[1].count);
  add(kEnergyPool, 0, p.pool.count);
  p.energy_chunks = c;
}

namespace {
// Batches from this size on run the dense pairwise terms with the instances on the lanes.
constexpr int64_t kLanesMinBatch = 16;
size_t partial_bytes(const Plan& p, int64_t B) {
  const size_t n = (size_t)std::max<int64_t>(1, B * p.energy_chunks) * sizeof(EnergyPartial);
  return (n + 255) & ~(size_t)255;
}
}  // namespace

size_t energy_workspace_bytes(const Plan& p, int64_t B) {
  size_t n = partial_bytes(p, B);
  if (B >= kLanesMinBatch && !p.pairwise.empty()) n += sizeof(int32_t) * (size_t)(p.num_variables * B);
  return n;
}

cudaError_t energy(const Plan& p, cudaStream_t s, int64_t B, const float* lp, int64_t lp_stride,
                   const float* ev, int64_t ev_stride, const int32_t* map, int64_t map_stride,
                   float* out, void* ws, size_t ws_bytes) {
  (void)ws_bytes;
  ProfileScope ps(kProfReadout, s);
  EnergyPartial* part = static_cast<EnergyPartial*>(ws);
  Args a;
  a.var_off = p.var_off;
  a.var_of_vs = p.var_of_vs;
  a.lp = lp;
  a.lps = lp_stride;
  a.ev = ev;
  a.evs = ev_stride;
  a.map = map;
  a.ms = map_stride;
  a.B = B;
  a.chunks = p.energy_chunks;
  a.gen = p.enum_generic;
  const unsigned gy = (unsigned)std::min<int64_t>(B, 65535);
  bool lanes = false;
  for (const EnergySeg& es : p.energy_segs) lanes |= es.kind == kEnergyPairwise;
  lanes = lanes && B >= kLanesMinBatch && lp != nullptr;
  int32_t* map_t = nullptr;
  if (lanes) {
    map_t = reinterpret_cast<int32_t*>(static_cast<char*>(ws) + partial_bytes(p, B));
    const dim3 tg((unsigned)((p.num_variables + 31) / 32), (unsigned)((B + 31) / 32));
    transpose_states_kernel<<<tg, dim3(32, 8), 0, s>>>(map, map_stride, p.num_variables, B, map_t);
  }
  for (size_t s0 = 0; s0 < p.energy_segs.size(); s0 += kMaxSegsPerLaunch) {
    Launch L;
    L.nseg = (int)std::min<size_t>(kMaxSegsPerLaunch, p.energy_segs.size() - s0);
    for (int k = 0; k < L.nseg; ++k) L.seg[k] = seg_dev(p, p.energy_segs[s0 + k]);
    const EnergySeg& last = p.energy_segs[s0 + L.nseg - 1];
    const int64_t first = p.energy_segs[s0].chunk_begin;
    const int64_t n = last.chunk_begin + chunks_of(last.items) - first;
    energy_partial_kernel<<<dim3((unsigned)n, gy), kEnergyThreads, 0, s>>>(a, L, first,
                                                                            lanes ? 1 : 0, part);
    if (lanes) {
      for (int k = 0; k < L.nseg; ++k) {
        const SegDev& d = L.seg[k];
        if (d.kind != kEnergyPairwise) continue;
        const dim3 g((unsigned)chunks_of(d.items), (unsigned)((B + 31) / 32));
        energy_pairwise_kernel<<<g, kEnergyThreads, 0, s>>>(a, d, map_t, part);
      }
    }
  }
  const int present = (p.num_enum_factors > 0 ? 1 : 0) | (p.logical[0].count > 0 ? 2 : 0) |
                      (p.logical[1].count > 0 ? 4 : 0) | (p.pool.count > 0 ? 8 : 0);
  const int64_t threads = B * 32;
  energy_final_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
      part, p.energy_chunks, B, (long long)p.num_enum_factors, present, out);
  return cudaGetLastError();
}

cudaError_t energy_terms(const Plan& p, cudaStream_t s, int64_t B, const float* ev,
                         int64_t ev_stride, const int32_t* map, int64_t map_stride, float* var_e,
                         int32_t* fac_cfg) {
  ProfileScope ps(kProfReadout, s);
  Args a{};
  a.var_off = p.var_off;
  a.var_of_vs = p.var_of_vs;
  a.ev = ev;
  a.evs = ev_stride;
  a.map = map;
  a.ms = map_stride;
  a.B = B;
  a.chunks = p.energy_chunks;
  a.gen = p.enum_generic;
  const unsigned gy = (unsigned)std::min<int64_t>(B, 65535);
  for (size_t s0 = 0; s0 < p.energy_segs.size(); s0 += kMaxSegsPerLaunch) {
    Launch L;
    L.nseg = (int)std::min<size_t>(kMaxSegsPerLaunch, p.energy_segs.size() - s0);
    for (int k = 0; k < L.nseg; ++k) L.seg[k] = seg_dev(p, p.energy_segs[s0 + k]);
    const EnergySeg& last = p.energy_segs[s0 + L.nseg - 1];
    const int64_t first = p.energy_segs[s0].chunk_begin;
    const int64_t n = last.chunk_begin + chunks_of(last.items) - first;
    energy_terms_kernel<<<dim3((unsigned)n, gy), kEnergyThreads, 0, s>>>(
        a, L, first, p.num_variables, p.num_factors, var_e, fac_cfg);
  }
  return cudaGetLastError();
}

}  // namespace pgbp
