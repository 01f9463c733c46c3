/* CPU oracle for loopy belief propagation: a float32 restatement of PGMax 0.6.1.
 *
 * TEST INFRASTRUCTURE ONLY (see bp_oracle.h). Compiled with -ffp-contract=off so that no
 * multiply-add is fused: each float32 operation rounds exactly as the reference's JAX ops do.
 * Scatter-adds / scatter-maxes run serially in index order, which is XLA:CPU's order and the order
 * of np.ufunc.at.
 *
 * Reference steps restated (paths relative to the PGMax source tree):
 *   normalize_and_clip_msgs ............ pgmax/infer/bp.py:222-260
 *   pass_var_to_fac_messages ........... pgmax/infer/bp.py:191-219
 *   run_with_diffs / update ............ pgmax/infer/bp.py:63-155
 *   pass_enum_fac_to_var_messages ...... pgmax/factor/enum.py:398-475
 *   pass_logical_fac_to_var_messages ... pgmax/factor/logical.py:492-779
 *   pass_pool_fac_to_var_messages ...... pgmax/factor/pool.py:276-474
 *   get_maxes_and_argmaxes, logsumexps_with_temp, log1mexp, logaddexp_with_temp,
 *   logminusexp_with_temp .............. pgmax/factor/update_utils.py:25-190
 *   constants MSG_NEG_INF, LOG_POTENTIAL_MAX_ABS, TEMPERATURE_STABILITY_THRE
 *                                        pgmax/utils/__init__.py:26-37, pgmax/factor/logical.py:33
 */
#include "bp_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define MSG_NEG_INF_F ((float)-1e32)
#define LOG_POT_MAX_ABS_F ((float)1e6)
#define STABILITY_THRE 0.5

/* numpy / XLA maximum and minimum: NaN-propagating, first argument kept on ties. */
static inline float fmaxp(float a, float b) { return (a >= b || a != a) ? a : b; }
static inline float fminp(float a, float b) { return (a <= b || a != a) ? a : b; }

/* T * log1p(exp((min - max) / T)) + max  (update_utils.py:150-166) */
static inline float logaddexp_t(float a, float b, float t) {
  float mx = fmaxp(a, b);
  float mn = fminp(a, b);
  float w = log1pf(expf((mn - mx) / t));
  return t * w + mx;
}

/* log(1 - exp(-x)) (update_utils.py:134-147); both branches evaluated as jnp.where does. */
static inline float log1mexp_f(float x) {
  float a = logf(-expm1f(-x));
  float b = log1pf(-expf(-x));
  return (x <= logf(2.0f)) ? a : b;
}

/* where(a >= b + eps, T * log1mexp((a - b) / T) + a, -inf) (update_utils.py:169-190) */
static inline float logminusexp_t(float a, float b, float t, float eps) {
  float v = t * log1mexp_f((a - b) / t) + a;
  return (a >= b + eps) ? v : -INFINITY;
}

/* JAX scatter index normalisation: negatives wrap once, out of range is dropped (-1). */
static inline int64_t norm_idx(int64_t i, int64_t n) {
  if (i < 0) i += n;
  return (i < 0 || i >= n) ? -1 : i;
}

static void normalize_and_clip(const bpo_wiring* w, float* msgs, float* max_by_edges) {
  const int64_t ne = w->num_edges, ns = w->num_edge_states;
  for (int64_t e = 0; e < ne; ++e) max_by_edges[e] = -INFINITY;
  for (int64_t i = 0; i < ns; ++i) {
    int32_t e = w->edge_indices_for_edge_states[i];
    max_by_edges[e] = fmaxp(max_by_edges[e], msgs[i]);
  }
  for (int64_t i = 0; i < ns; ++i) {
    float v = msgs[i] - max_by_edges[w->edge_indices_for_edge_states[i]];
    msgs[i] = fmaxp(v, MSG_NEG_INF_F);
  }
}

static void var_to_fac(const bpo_wiring* w, const float* ftov, const float* evidence,
                       float* var_sums, float* vtof) {
  memcpy(var_sums, evidence, sizeof(float) * (size_t)w->num_var_states);
  for (int64_t i = 0; i < w->num_edge_states; ++i)
    var_sums[w->var_states_for_edge_states[i]] += ftov[i];
  for (int64_t i = 0; i < w->num_edge_states; ++i)
    vtof[i] = var_sums[w->var_states_for_edge_states[i]] - ftov[i];
}

/* ------------------------------------------------------------------------------------- Enum */
static int enum_update(const bpo_wiring* w, const float* vtof, int64_t n_es, const float* lp,
                       double temperature, float* out) {
  const int64_t nr = w->enum_num_rows, nc = w->enum_num_val_configs;
  const int32_t* ci = w->enum_factor_configs_indices;
  const int32_t* ce = w->enum_factor_configs_edge_states;
  float* summary = (float*)calloc((size_t)(nc > 0 ? nc : 1), sizeof(float));
  float* maxes = (float*)malloc(sizeof(float) * (size_t)(n_es > 0 ? n_es : 1));
  if (!summary || !maxes) { free(summary); free(maxes); return 1; }
  for (int64_t r = 0; r < nr; ++r) summary[ci[r]] += vtof[ce[r]];
  for (int64_t c = 0; c < nc; ++c) summary[c] = summary[c] + lp[c];
  for (int64_t e = 0; e < n_es; ++e) maxes[e] = -INFINITY;
  for (int64_t r = 0; r < nr; ++r) maxes[ce[r]] = fmaxp(maxes[ce[r]], summary[ci[r]]);
  if (temperature == 0.0) {
    for (int64_t e = 0; e < n_es; ++e) out[e] = maxes[e];
  } else {
    const float t = (float)temperature;
    for (int64_t e = 0; e < n_es; ++e) out[e] = 0.0f;
    for (int64_t r = 0; r < nr; ++r) out[ce[r]] += expf((summary[ci[r]] - maxes[ce[r]]) / t);
    for (int64_t e = 0; e < n_es; ++e) out[e] = t * logf(out[e]) + maxes[e];
  }
  for (int64_t e = 0; e < n_es; ++e) out[e] = out[e] - vtof[e];
  free(summary);
  free(maxes);
  return 0;
}

/* get_maxes_and_argmaxes (update_utils.py:25-64): the argmax is the LAST index attaining the max. */
static void maxes_argmaxes(const float* data, const int32_t* labels, int64_t n, int64_t nl,
                           float* maxes, int64_t* argmaxes) {
  for (int64_t f = 0; f < nl; ++f) { maxes[f] = -INFINITY; argmaxes[f] = INT32_MIN; }
  for (int64_t i = 0; i < n; ++i) maxes[labels[i]] = fmaxp(maxes[labels[i]], data[i]);
  for (int64_t i = 0; i < n; ++i) {
    int64_t pos = (int64_t)(int32_t)(i - (data[i] != maxes[labels[i]] ? n : 0));
    if (pos > argmaxes[labels[i]]) argmaxes[labels[i]] = pos;
  }
}

/* -------------------------------------------------------------------------------- OR / AND */
static int logical_update(const bpo_wiring* w, int which, const float* vtof, int64_t n_es,
                          double temperature, int normalize, float* out) {
  const int64_t P = w->logical_num_parents[which], F = w->logical_num_factors[which];
  const int32_t* pfi = w->logical_parents_factor_indices[which];
  const int32_t* pmi = w->logical_parents_msg_indices[which];
  const int32_t* ch = w->logical_children_edge_states[which];
  const int off = which == 0 ? 1 : -1;
  const float t = (float)temperature;
  size_t np_ = (size_t)(P > 0 ? P : 1), nf_ = (size_t)(F > 0 ? F : 1);
  float* buf = (float*)malloc(sizeof(float) * (np_ * 10 + nf_ * 10));
  int64_t* arg1 = (int64_t*)malloc(sizeof(int64_t) * nf_);
  int64_t* nump = (int64_t*)calloc(nf_, sizeof(int64_t));
  if (!buf || !arg1 || !nump) { free(buf); free(arg1); free(nump); return 1; }
  float *p_rel = buf, *p_oth = p_rel + np_, *p_diff = p_oth + np_, *p_msg_rel = p_diff + np_,
        *p_msg_oth = p_msg_rel + np_, *tmp1 = p_msg_oth + np_, *tmp2 = tmp1 + np_,
        *opt1 = tmp2 + np_, *opt2 = opt1 + np_, *wo = opt2 + np_;
  float *c_rel = wo + np_, *c_oth = c_rel + nf_, *fs_oth = c_oth + nf_, *max1 = fs_oth + nf_,
        *max2 = max1 + nf_, *fs_x = max2 + nf_, *ch_rel = fs_x + nf_;

  for (int64_t i = 0; i < P; ++i) {
    p_rel[i] = vtof[pmi[i] + off];
    p_oth[i] = vtof[pmi[i]];
    p_diff[i] = p_rel[i] - p_oth[i];
  }
  for (int64_t f = 0; f < F; ++f) {
    c_rel[f] = vtof[ch[f] + off];
    c_oth[f] = vtof[ch[f]];
    fs_oth[f] = 0.0f;
  }
  for (int64_t i = 0; i < P; ++i) fs_oth[pfi[i]] += p_oth[i];
  maxes_argmaxes(p_diff, pfi, P, F, max1, arg1);
  memcpy(wo, p_diff, sizeof(float) * (size_t)P);
  for (int64_t f = 0; f < F; ++f) {
    int64_t a = norm_idx(arg1[f], P);
    if (a >= 0) wo[a] = -INFINITY;
  }
  for (int64_t f = 0; f < F; ++f) max2[f] = -INFINITY;
  for (int64_t i = 0; i < P; ++i) max2[pfi[i]] = fmaxp(max2[pfi[i]], wo[i]);

  if (temperature == 0.0) {
    /* logical.py:598-643 */
    float* mx = tmp1;
    for (int64_t i = 0; i < P; ++i) mx[i] = fmaxp(p_oth[i], p_rel[i]);
    for (int64_t f = 0; f < F; ++f) fs_x[f] = 0.0f;
    for (int64_t i = 0; i < P; ++i) fs_x[pfi[i]] += mx[i];
    for (int64_t i = 0; i < P; ++i) p_msg_rel[i] = (fs_x[pfi[i]] + c_rel[pfi[i]]) - mx[i];
    for (int64_t f = 0; f < F; ++f) {
      float m0 = fminp(0.0f, max1[f]);
      ch_rel[f] = fs_x[f] + m0;
    }
    for (int64_t i = 0; i < P; ++i) {
      int32_t f = pfi[i];
      opt1[i] = (c_oth[f] + fs_oth[f]) - p_oth[i];
      opt2[i] = p_msg_rel[i] + fminp(0.0f, max1[f]);
    }
    for (int64_t f = 0; f < F; ++f) {
      int64_t a = norm_idx(arg1[f], P);
      if (a >= 0) opt2[a] = p_msg_rel[a] + fminp(0.0f, max2[f]);
    }
    for (int64_t i = 0; i < P; ++i) p_msg_oth[i] = fmaxp(opt1[i], opt2[i]);
  } else {
    /* logical.py:645-737 */
    float* lse = tmp1;
    float* fs_oth_wo = tmp2;
    for (int64_t i = 0; i < P; ++i) lse[i] = logaddexp_t(p_rel[i], p_oth[i], t);
    for (int64_t f = 0; f < F; ++f) fs_x[f] = 0.0f;
    for (int64_t i = 0; i < P; ++i) fs_x[pfi[i]] += lse[i];
    for (int64_t i = 0; i < P; ++i) {
      int32_t f = pfi[i];
      float fs_lse_wo = fs_x[f] - lse[i];
      fs_oth_wo[i] = fs_oth[f] - p_oth[i];
      p_msg_rel[i] = c_rel[f] + fs_lse_wo;
      opt2[i] = c_rel[f] + fs_lse_wo;  /* option 2 */
      opt1[i] = c_oth[f] + fs_oth_wo[i];
    }
    const float eps4 = (float)1e-4;
    for (int64_t f = 0; f < F; ++f) ch_rel[f] = logminusexp_t(fs_x[f], fs_oth[f], t, eps4);
    if (temperature < STABILITY_THRE) {
      for (int64_t f = 0; f < F; ++f) {
        float lb = logaddexp_t(fs_oth[f] + max1[f], fs_oth[f] + max2[f], t);
        ch_rel[f] = fmaxp(ch_rel[f], lb);
      }
    }
    for (int64_t i = 0; i < P; ++i) {
      int32_t f = pfi[i];
      float opt3 = c_rel[f] + fs_oth_wo[i];
      float la12 = logaddexp_t(opt1[i], opt2[i], t);
      p_msg_oth[i] = logminusexp_t(la12, opt3, t, eps4);
    }
    if (temperature < STABILITY_THRE) {
      float* fsp = wo; /* reuse: factorsum_parents_other_plus_max_diff_wo_self */
      for (int64_t i = 0; i < P; ++i) fsp[i] = fs_oth_wo[i] + max1[pfi[i]];
      for (int64_t f = 0; f < F; ++f) {
        int64_t a = norm_idx(arg1[f], P);
        if (a >= 0) fsp[a] = fs_oth_wo[a] + max2[f];
      }
      for (int64_t i = 0; i < P; ++i) {
        int32_t f = pfi[i];
        float lb = logaddexp_t(opt1[i], c_rel[f] + fsp[i], t);
        p_msg_oth[i] = fmaxp(p_msg_oth[i], lb);
      }
    }
  }
  /* single-parent factors (logical.py:739-757) */
  for (int64_t i = 0; i < P; ++i) nump[pfi[i]] += 1;
  {
    int64_t first = 0;
    for (int64_t f = 0; f < F; ++f) {
      int64_t a = norm_idx(first, P);
      if (nump[f] == 1 && a >= 0) {
        p_msg_rel[a] = c_rel[f];
        p_msg_oth[a] = c_oth[f];
      }
      first += nump[f];
    }
  }
  for (int64_t e = 0; e < n_es; ++e) out[e] = 0.0f;
  if (normalize) {
    for (int64_t i = 0; i < P; ++i) out[pmi[i] + off] = p_msg_rel[i] - p_msg_oth[i];
    for (int64_t f = 0; f < F; ++f) out[ch[f] + off] = ch_rel[f] - fs_oth[f];
  } else {
    for (int64_t i = 0; i < P; ++i) out[pmi[i] + off] = p_msg_rel[i];
    for (int64_t i = 0; i < P; ++i) out[pmi[i]] = p_msg_oth[i];
    for (int64_t f = 0; f < F; ++f) out[ch[f] + off] = ch_rel[f];
    for (int64_t f = 0; f < F; ++f) out[ch[f]] = fs_oth[f];
  }
  free(buf);
  free(arg1);
  free(nump);
  return 0;
}

/* ------------------------------------------------------------------------------------ Pool */
static int pool_update(const bpo_wiring* w, const float* vtof, int64_t n_es, double temperature,
                       int normalize, float* out) {
  const int64_t P = w->pool_num_choices, F = w->pool_num_factors;
  const int32_t* cfi = w->pool_choices_factor_indices;
  const int32_t* cmi = w->pool_choices_msg_indices;
  const int32_t* ind = w->pool_indicators_edge_states;
  const float t = (float)temperature;
  size_t np_ = (size_t)(P > 0 ? P : 1), nf_ = (size_t)(F > 0 ? F : 1);
  float* buf = (float*)malloc(sizeof(float) * (np_ * 6 + nf_ * 8));
  int64_t* arg1 = (int64_t*)malloc(sizeof(int64_t) * nf_);
  int64_t* num = (int64_t*)calloc(nf_, sizeof(int64_t));
  if (!buf || !arg1 || !num) {
    free(buf); free(arg1); free(num);
    return 1;
  }
  float *pc_diff = buf, *pc_zero = pc_diff + np_, *pc_ones = pc_zero + np_,
        *pc_mdiff = pc_ones + np_, *wo = pc_mdiff + np_, *tmp = wo + np_;
  float *pi_diff = tmp + np_, *pi_one = pi_diff + nf_, *sums0 = pi_one + nf_, *max1 = sums0 + nf_,
        *max2 = max1 + nf_, *pi_mdiff = max2 + nf_, *fl = pi_mdiff + nf_, *am = fl + nf_;

  for (int64_t i = 0; i < P; ++i) {
    pc_diff[i] = vtof[cmi[i] + 1] - vtof[cmi[i]];
    pc_zero[i] = vtof[cmi[i]];
  }
  for (int64_t f = 0; f < F; ++f) {
    pi_diff[f] = vtof[ind[f] + 1] - vtof[ind[f]];
    pi_one[f] = vtof[ind[f] + 1];
    sums0[f] = 0.0f;
  }
  for (int64_t i = 0; i < P; ++i) sums0[cfi[i]] += pc_zero[i];
  for (int64_t i = 0; i < P; ++i) pc_ones[i] = (sums0[cfi[i]] + pi_one[cfi[i]]) - pc_zero[i];
  maxes_argmaxes(pc_diff, cfi, P, F, max1, arg1);

  if (temperature == 0.0) {
    /* pool.py:365-388 */
    memcpy(wo, pc_diff, sizeof(float) * (size_t)P);
    for (int64_t f = 0; f < F; ++f) {
      int64_t a = norm_idx(arg1[f], P);
      if (a >= 0) wo[a] = -INFINITY;
    }
    for (int64_t f = 0; f < F; ++f) max2[f] = -INFINITY;
    for (int64_t i = 0; i < P; ++i) max2[cfi[i]] = fmaxp(max2[cfi[i]], wo[i]);
    for (int64_t i = 0; i < P; ++i) pc_mdiff[i] = fminp(pi_diff[cfi[i]], -max1[cfi[i]]);
    for (int64_t f = 0; f < F; ++f) {
      int64_t a = norm_idx(arg1[f], P);
      if (a >= 0) pc_mdiff[a] = fminp(pi_diff[f], -max2[f]);
    }
    for (int64_t f = 0; f < F; ++f) pi_mdiff[f] = max1[f];
  } else {
    /* pool.py:390-428 */
    float* sumexp = fl;
    for (int64_t f = 0; f < F; ++f) sumexp[f] = 0.0f;
    for (int64_t i = 0; i < P; ++i) sumexp[cfi[i]] += expf((pc_diff[i] - max1[cfi[i]]) / t);
    for (int64_t f = 0; f < F; ++f) pi_mdiff[f] = t * logf(sumexp[f]) + max1[f];
    for (int64_t f = 0; f < F; ++f) fl[f] = logaddexp_t(pi_mdiff[f], -pi_diff[f], t);
    const float eps30 = (float)1e-30;
    for (int64_t i = 0; i < P; ++i) pc_mdiff[i] = -logminusexp_t(fl[cfi[i]], pc_diff[i], t, eps30);
    memcpy(wo, pc_diff, sizeof(float) * (size_t)P);
    for (int64_t f = 0; f < F; ++f) {
      int64_t a = norm_idx(arg1[f], P);
      if (a >= 0) wo[a] = -pi_diff[f];
    }
    /* -logsumexps_with_temp(wo) with its own maxes */
    for (int64_t f = 0; f < F; ++f) max2[f] = -INFINITY;
    for (int64_t i = 0; i < P; ++i) max2[cfi[i]] = fmaxp(max2[cfi[i]], wo[i]);
    for (int64_t f = 0; f < F; ++f) am[f] = 0.0f;
    for (int64_t i = 0; i < P; ++i) am[cfi[i]] += expf((wo[i] - max2[cfi[i]]) / t);
    for (int64_t f = 0; f < F; ++f) am[f] = -(t * logf(am[f]) + max2[f]);
    for (int64_t f = 0; f < F; ++f) {
      int64_t a = norm_idx(arg1[f], P);
      if (a >= 0) pc_mdiff[a] = am[f];
    }
  }
  /* single-choice factors (pool.py:430-450) */
  for (int64_t i = 0; i < P; ++i) num[cfi[i]] += 1;
  {
    int64_t first = 0;
    for (int64_t f = 0; f < F; ++f) {
      int64_t a = norm_idx(first, P);
      if (num[f] == 1 && a >= 0) {
        pc_mdiff[a] = pi_diff[f];
        pc_ones[a] = pi_one[f];
      }
      first += num[f];
    }
  }
  for (int64_t e = 0; e < n_es; ++e) out[e] = 0.0f;
  if (normalize) {
    for (int64_t i = 0; i < P; ++i) out[cmi[i] + 1] = pc_mdiff[i];
    for (int64_t f = 0; f < F; ++f) out[ind[f] + 1] = pi_mdiff[f];
  } else {
    for (int64_t i = 0; i < P; ++i) out[cmi[i] + 1] = pc_ones[i];
    for (int64_t i = 0; i < P; ++i) out[cmi[i]] = pc_ones[i] - pc_mdiff[i];
    for (int64_t f = 0; f < F; ++f) out[ind[f] + 1] = sums0[f] + pi_mdiff[f];
    for (int64_t f = 0; f < F; ++f) out[ind[f]] = sums0[f];
  }
  free(buf);
  free(arg1);
  free(num);
  return 0;
}

int bpo_factor_update(const bpo_wiring* w, int type, const float* vtof, const float* lp,
                      double temperature, int normalize, float* out) {
  if (type < 0 || type > 3) return 2;
  const int64_t n_es = w->msgs_range[type][1] - w->msgs_range[type][0];
  switch (type) {
    case 0: return enum_update(w, vtof, n_es, lp, temperature, out);
    case 1: return logical_update(w, 0, vtof, n_es, temperature, normalize, out);
    case 2: return logical_update(w, 1, vtof, n_es, temperature, normalize, out);
    default: return pool_update(w, vtof, n_es, temperature, normalize, out);
  }
}

int bpo_run(const bpo_wiring* w, const float* log_potentials, const float* evidence,
            const float* msgs_in, int64_t num_iters, double damping, double temperature,
            float* msgs_out, float* deltas) {
  const int64_t ns = w->num_edge_states;
  int64_t np_ = w->potentials_range[3][1];
  for (int t = 0; t < 4; ++t)
    if (w->potentials_range[t][1] > np_) np_ = w->potentials_range[t][1];
  size_t nsz = (size_t)(ns > 0 ? ns : 1);
  float* lp = (float*)malloc(sizeof(float) * (size_t)(np_ > 0 ? np_ : 1));
  float* msgs = (float*)malloc(sizeof(float) * nsz);
  float* vtof = (float*)malloc(sizeof(float) * nsz);
  float* ftov = (float*)malloc(sizeof(float) * nsz);
  float* sums = (float*)malloc(sizeof(float) * (size_t)(w->num_var_states > 0 ? w->num_var_states : 1));
  float* mbe = (float*)malloc(sizeof(float) * (size_t)(w->num_edges > 0 ? w->num_edges : 1));
  int rc = 0;
  if (!lp || !msgs || !vtof || !ftov || !sums || !mbe) { rc = 1; goto done; }
  /* bp.py:85-87 */
  for (int64_t i = 0; i < np_; ++i)
    lp[i] = fminp(fmaxp(log_potentials[i], -LOG_POT_MAX_ABS_F), LOG_POT_MAX_ABS_F);
  memcpy(msgs, msgs_in, sizeof(float) * (size_t)ns);
  normalize_and_clip(w, msgs, mbe);
  {
    const float d = (float)damping;
    const float omd = (float)(1.0 - damping);
    const int64_t iters = num_iters > 1 ? num_iters : 1;
    for (int64_t it = 0; it < iters; ++it) {
      var_to_fac(w, msgs, evidence, sums, vtof);
      for (int64_t i = 0; i < ns; ++i) ftov[i] = 0.0f;
      for (int type = 0; type < 4; ++type) {
        const int64_t ms = w->msgs_range[type][0], me = w->msgs_range[type][1];
        if (ms == me) continue;
        rc = bpo_factor_update(w, type, vtof + ms, lp + w->potentials_range[type][0], temperature,
                               1, ftov + ms);
        if (rc) goto done;
      }
      for (int64_t i = 0; i < ns; ++i) ftov[i] = d * msgs[i] + omd * ftov[i];
      normalize_and_clip(w, ftov, mbe);
      float delta = -INFINITY;
      for (int64_t i = 0; i < ns; ++i) {
        float a = fabsf(ftov[i] - msgs[i]);
        delta = fmaxp(delta, a);
      }
      deltas[it] = delta;
      float* sw = msgs; msgs = ftov; ftov = sw;
    }
  }
  memcpy(msgs_out, msgs, sizeof(float) * (size_t)ns);
done:
  free(lp); free(msgs); free(vtof); free(ftov); free(sums); free(mbe);
  return rc;
}

int bpo_run_batch(const bpo_wiring* w, int64_t batch, const float* log_potentials,
                  int64_t lp_stride, const float* evidence, int64_t ev_stride,
                  const float* msgs_in, int64_t msgs_stride, int64_t num_iters, double damping,
                  double temperature, float* msgs_out, float* deltas, int num_threads) {
  const int64_t nd = num_iters > 1 ? num_iters : 1;
  int rc = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(num_threads) reduction(| : rc)
  for (int64_t b = 0; b < batch; ++b) {
    rc |= bpo_run(w, log_potentials + b * lp_stride, evidence + b * ev_stride,
                  msgs_in + b * msgs_stride, num_iters, damping, temperature,
                  msgs_out + b * w->num_edge_states, deltas + b * nd);
  }
  return rc;
}

int bpo_beliefs(const bpo_wiring* w, const float* evidence, const float* msgs, float* beliefs) {
  memcpy(beliefs, evidence, sizeof(float) * (size_t)w->num_var_states);
  for (int64_t i = 0; i < w->num_edge_states; ++i)
    beliefs[w->var_states_for_edge_states[i]] += msgs[i];
  return 0;
}

/* ---- the Gumbel stream of perturb-and-MAP runs (bpo_gumbel, see bp_oracle.h) */
static uint64_t g_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* ln(x) for a positive normal float: x = m 2^e with m in [sqrt(2)/2, sqrt(2)], then
 * ln(m) = 2 atanh((m - 1) / (m + 1)) by its series up to the z^4 / 9 term. */
static float g_ln(float x) {
  uint32_t bits;
  memcpy(&bits, &x, sizeof(bits));
  int e = (int)((bits >> 23) & 0xffu) - 127;
  const uint32_t mb = (bits & 0x007fffffu) | 0x3f800000u;
  float m;
  memcpy(&m, &mb, sizeof(m));
  if (m > 0x1.6a09e6p+0f) {
    m = m * 0.5f;
    e += 1;
  }
  const float s = (m - 1.0f) / (m + 1.0f);
  const float z = s * s;
  float p = 0x1.c71c72p-4f;
  p = p * z + 0x1.24924ap-3f;
  p = p * z + 0x1.99999ap-3f;
  p = p * z + 0x1.555556p-2f;
  p = p * z + 1.0f;
  const float lm = (s * p) * 2.0f;
  return (float)e * 0x1.62e430p-1f + lm;
}

void bpo_gumbel(uint64_t seed, int64_t first, int64_t count, float* out) {
  const uint64_t key = g_mix64(seed);
  for (int64_t i = 0; i < count; ++i) {
    const uint64_t c = (uint64_t)(first + i);
    const uint64_t r = g_mix64(key + (c + 1ull) * 0x9E3779B97F4A7C15ull);
    const uint32_t k = (uint32_t)(r >> 41);
    const float u = (float)(2u * k + 1u) * 0x1.0p-24f;
    const float w = -g_ln(u);
    out[i] = -g_ln(w);
  }
}
