// Per-step linearisation of a model f: R^DIN -> R^DOUT with additive noise
// q ~ N(qm, qc qc^T) around x ~ N(m, C C^T), returning (F, L, b) with
// f(x') + q ~= F x' + b + N(0, L L^T).
#pragma once
#include "ss_models.cuh"

namespace ss {

// Unit sigma point k of the rule (xi, DIN) with its weights.
template <typename R, int DIN, int METHOD>
SS_DEV void sigma_point(const RuleArgs& ru, int k, R (&xi)[DIN], R& wm, R& wc) {
  SS_UNROLL
  for (int j = 0; j < DIN; ++j) xi[j] = R(0);
  if constexpr (METHOD == SS_LIN_CUBATURE) {
    // +-sqrt(n) e_j, weights 1/(2n) (parsmooth/linearization/_cubature.py:63-85)
    const R sc = ss_sqrt(R(DIN));
    SS_UNROLL
    for (int j = 0; j < DIN; ++j) xi[j] = (k == j) ? sc : ((k == j + DIN) ? -sc : R(0));
    wm = wc = R(1) / R(2 * DIN);
  } else if constexpr (METHOD == SS_LIN_UNSCENTED) {
    // 0, +-sqrt(n + lambda) e_j (parsmooth/linearization/_unscented.py:42-101)
    const R sc = rule_ut<R>(ru, 0);
    SS_UNROLL
    for (int j = 0; j < DIN; ++j) xi[j] = (k == j + 1) ? sc : ((k == j + 1 + DIN) ? -sc : R(0));
    wm = (k == 0) ? rule_ut<R>(ru, 1) : rule_ut<R>(ru, 3);
    wc = (k == 0) ? rule_ut<R>(ru, 2) : rule_ut<R>(ru, 3);
  } else {
    // tensor-product Gauss-Hermite: dimension j takes root (k / p^j) % p
    // (parsmooth/linearization/_gh.py:73-126)
    const int p = ru.gh_order;
    int rem = k;
    R w = R(1);
    SS_UNROLL
    for (int j = 0; j < DIN; ++j) {
      const int d = rem % p;
      rem /= p;
      xi[j] = rule_gh_root<R>(ru, d);
      w *= rule_gh_w<R>(ru, d);
    }
    wm = wc = w;
  }
}

template <int DIN, int METHOD>
SS_DEV int num_points(const RuleArgs& ru) {
  if constexpr (METHOD == SS_LIN_CUBATURE) return 2 * DIN;
  else if constexpr (METHOD == SS_LIN_UNSCENTED) return 2 * DIN + 1;
  else {
    int n = 1;
    for (int j = 0; j < DIN; ++j) n *= ru.gh_order;
    return n;
  }
}

// SLR forms: DOWNDATE follows parsmooth/linearization/_sigma_points.py:63-79
// literally (tria of the weighted deviations and the noise factor, then DIN
// rank-1 downdates by the columns of F C).  RESIDUAL streams the weighted
// regression residuals d_k - S xi_k, which have the same second moment
// (Phi + Q - F P F^T) whenever the rule reproduces the identity covariance,
// and avoids the cancellation of the downdate in FP32.
enum { SS_SLR_DOWNDATE = 1, SS_SLR_RESIDUAL = 2 };

// Symmetric rules (cubature, unscented) with the model evaluated once per
// point.  Point k = 0 is the unscented centre; points (+j, -j) are
// m +- sc C[:, j].  With f_j^+- = f(m +- sc C[:, j]):
//   S[:, j] = w sc (f_j^+ - f_j^-)                       (so that F = S C^{-1})
//   residual of both points of pair j:  (f_j^+ + f_j^-)/2 - m_f
// so the residual form needs one column sqrt(2w) ((f^+ + f^-)/2 - m_f) per
// pair (plus the centre's sqrt(wc0) (f_0 - m_f)), and the downdate form the
// 2n(+1) columns sqrt(wc_k) (f_k - m_f).  Either matrix is triangularised by
// one Householder tria.
template <typename R, int DIN, int DOUT, class Fn, int METHOD>
SS_DEV void linearize_symmetric(const Fn& f, const R (&m)[DIN], const R (&C)[DIN][DIN], const R (&qm)[DOUT],
                                const R (&qc)[DOUT][DOUT], const RuleArgs& ru, int slr_form,
                                R (&F)[DOUT][DIN], R (&L)[DOUT][DOUT], R (&b)[DOUT]) {
  constexpr bool UT = (METHOD == SS_LIN_UNSCENTED);
  constexpr int NC = UT ? 1 : 0;  // centre point
  R sc, w, wm0 = R(0), wc0 = R(0);
  if constexpr (UT) {
    sc = rule_ut<R>(ru, 0);
    wm0 = rule_ut<R>(ru, 1);
    wc0 = rule_ut<R>(ru, 2);
    w = rule_ut<R>(ru, 3);
  } else {
    sc = ss_sqrt(R(DIN));
    w = R(1) / R(2 * DIN);
  }
  // conditional-moments models (parsmooth/linearization/_sigma_points.py:25-60): the noise
  // columns are the points' weighted conditional factors sqrt(wc_k) chol(Cov[y | x_k])
  constexpr bool COND = IsConditional<Fn>::value;
  constexpr int NQ = COND ? (NC + 2 * DIN) * DOUT : DOUT;   // noise columns
  constexpr int NCP = COND ? DIN : 1;                       // stored conditional factors
  R fp[DIN][DOUT], fn[DIN][DOUT], f0[DOUT];
  R cp[NCP][DOUT][DOUT], cn[NCP][DOUT][DOUT], c0[DOUT][DOUT];
  if constexpr (UT) {
    f.eval(m, f0);
    if constexpr (COND) f.cond_chol(m, c0);
  }
  SS_UNROLL
  for (int j = 0; j < DIN; ++j) {
    R xp[DIN], xn[DIN];
    SS_UNROLL
    for (int i = 0; i < DIN; ++i) {
      // C is lower triangular: coordinates above column j stay exactly at the mean,
      // so model outputs that depend only on those coordinates are shared by the
      // points (the compiler evaluates them once)
      const R d = sc * C[i][j];
      xp[i] = (i >= j) ? m[i] + d : m[i];
      xn[i] = (i >= j) ? m[i] - d : m[i];
    }
    f.eval(xp, fp[j]);
    f.eval(xn, fn[j]);
    if constexpr (COND) {
      f.cond_chol(xp, cp[j]);
      f.cond_chol(xn, cn[j]);
    }
  }
  // noise column q of output row i
  auto noise_col = [&](int i, int q) -> R {
    if constexpr (COND) {
      const int k = q / DOUT, jj = q - k * DOUT;   // point k: [centre], +0, -0, +1, -1, ...
      if constexpr (UT) {
        if (k == 0) return ss_sqrt(wc0) * c0[i][jj];
      }
      const int pk = k - NC;
      const int j = pk >> 1;
      const R sw = ss_sqrt(w);
      return (pk & 1) ? sw * cn[j][i][jj] : sw * cp[j][i][jj];
    } else {
      return qc[i][q];
    }
  };
  R mf[DOUT];
  SS_UNROLL
  for (int i = 0; i < DOUT; ++i) {
    R s = R(0);
    SS_UNROLL
    for (int j = 0; j < DIN; ++j) s += fp[j][i] + fn[j][i];
    mf[i] = w * s;
    if constexpr (UT) mf[i] += wm0 * f0[i];
  }
  R S[DOUT][DIN];
  SS_UNROLL
  for (int i = 0; i < DOUT; ++i) {
    SS_UNROLL
    for (int j = 0; j < DIN; ++j) S[i][j] = w * sc * (fp[j][i] - fn[j][i]);
  }
  // F^T = C^{-T} S^T
  {
    R Ft[DIN][DOUT];
    SS_UNROLL
    for (int i = 0; i < DIN; ++i) {
      SS_UNROLL
      for (int j = 0; j < DOUT; ++j) Ft[i][j] = S[j][i];
    }
    solve_lower_T<R, DIN, DOUT>(C, Ft);
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) {
      SS_UNROLL
      for (int j = 0; j < DIN; ++j) F[i][j] = Ft[j][i];
    }
  }
  if (slr_form == SS_SLR_RESIDUAL) {
    constexpr int NCOL = NC + DIN + NQ;
    R M[DOUT][NCOL];
    const R s2w = ss_sqrt(R(2) * w);
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) {
      if constexpr (UT) M[i][0] = ss_sqrt(wc0) * (f0[i] - mf[i]);
      SS_UNROLL
      for (int j = 0; j < DIN; ++j) M[i][NC + j] = s2w * (R(0.5) * (fp[j][i] + fn[j][i]) - mf[i]);
      SS_UNROLL
      for (int q = 0; q < NQ; ++q) M[i][NC + DIN + q] = noise_col(i, q);
    }
    // the noise block is the lower-triangular noise factor unless it is conditional
    typedef typename std::conditional<COND, PatFull, PatBlocks<DOUT, NC + DIN>>::type Pat;
    tria_sp<R, DOUT, NCOL, Pat>(M);
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) {
      SS_UNROLL
      for (int j = 0; j < DOUT; ++j) L[i][j] = (j <= i) ? M[i][j] : R(0);
    }
  } else {
    constexpr int NCOL = NC + 2 * DIN + NQ;
    R M[DOUT][NCOL];
    const R sw = ss_sqrt(w);
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) {
      if constexpr (UT) M[i][0] = ss_sqrt(wc0) * (f0[i] - mf[i]);
      SS_UNROLL
      for (int j = 0; j < DIN; ++j) {
        M[i][NC + j] = sw * (fp[j][i] - mf[i]);
        M[i][NC + DIN + j] = sw * (fn[j][i] - mf[i]);
      }
      SS_UNROLL
      for (int q = 0; q < NQ; ++q) M[i][NC + 2 * DIN + q] = noise_col(i, q);
    }
    typedef typename std::conditional<COND, PatFull, PatBlocks<DOUT, NC + 2 * DIN>>::type Pat;
    tria_sp<R, DOUT, NCOL, Pat>(M);
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) {
      SS_UNROLL
      for (int j = 0; j < DOUT; ++j) L[i][j] = (j <= i) ? M[i][j] : R(0);
    }
    // downdate by the columns of F C (= S)
    SS_UNROLL
    for (int j = 0; j < DIN; ++j) {
      R col[DOUT];
      SS_UNROLL
      for (int i = 0; i < DOUT; ++i) col[i] = S[i][j];
      chol_update<R, DOUT>(L, col, R(-1));
    }
  }
  SS_UNROLL
  for (int i = 0; i < DOUT; ++i) {
    R s = COND ? mf[i] : mf[i] + qm[i];
    SS_UNROLL
    for (int j = 0; j < DIN; ++j) s -= F[i][j] * m[j];
    b[i] = s;
  }
}

template <typename R, int DIN, int DOUT, class Fn, int METHOD>
SS_DEV void linearize(const Fn& f, const R (&m)[DIN], const R (&C)[DIN][DIN], const R (&qm)[DOUT],
                      const R (&qc)[DOUT][DOUT], const RuleArgs& ru, int slr_form,
                      R (&F)[DOUT][DIN], R (&L)[DOUT][DOUT], R (&b)[DOUT]) {
  if constexpr (METHOD == SS_LIN_EXTENDED) {
    // parsmooth/linearization/_extended.py:59-70: F = df/dx(m), L = qc, b = f(m) - F m + qm
    // (conditional models, _extended.py:43-56: chol = chol(Cov[y | m]), b = E[y | m] - F m)
    constexpr bool COND = IsConditional<Fn>::value;
    f.jac(m, F);
    R fm[DOUT];
    f.eval(m, fm);
    R cm[DOUT][DOUT];
    if constexpr (COND) f.cond_chol(m, cm);
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) {
      R s = COND ? fm[i] : fm[i] + qm[i];
      SS_UNROLL
      for (int j = 0; j < DIN; ++j) s -= F[i][j] * m[j];
      b[i] = s;
      SS_UNROLL
      for (int j = 0; j < DOUT; ++j) L[i][j] = COND ? cm[i][j] : qc[i][j];
    }
  } else if constexpr (METHOD == SS_LIN_CUBATURE || METHOD == SS_LIN_UNSCENTED) {
    linearize_symmetric<R, DIN, DOUT, Fn, METHOD>(f, m, C, qm, qc, ru, slr_form, F, L, b);
  } else {
    // Gauss-Hermite: p^n points streamed (recomputed per pass) with Givens updates
    const int np = num_points<DIN, METHOD>(ru);
    // pass 1: m_f = sum_k wm_k f(m + C xi_k)
    R mf[DOUT];
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) mf[i] = R(0);
#pragma unroll 1
    for (int k = 0; k < np; ++k) {
      R xi[DIN], x[DIN], fx[DOUT], wm, wc;
      sigma_point<R, DIN, METHOD>(ru, k, xi, wm, wc);
      SS_UNROLL
      for (int i = 0; i < DIN; ++i) {
        R s = m[i];
        SS_UNROLL
        for (int j = 0; j <= i; ++j) s += C[i][j] * xi[j];
        x[i] = s;
      }
      f.eval(x, fx);
      SS_UNROLL
      for (int i = 0; i < DOUT; ++i) mf[i] += wm * fx[i];
    }
    // pass 2: S = sum_k wc_k (f_k - m_f) xi_k^T; so that Psi_x = C S^T and F = S C^{-1}
    R S[DOUT][DIN];
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) {
      SS_UNROLL
      for (int j = 0; j < DIN; ++j) S[i][j] = R(0);
      SS_UNROLL
      for (int j = 0; j < DOUT; ++j) L[i][j] = R(0);
    }
    const bool residual = (slr_form == SS_SLR_RESIDUAL);
    if (!residual) {
#pragma unroll 1
      for (int k = 0; k < np; ++k) {
        R xi[DIN], x[DIN], fx[DOUT], wm, wc;
        sigma_point<R, DIN, METHOD>(ru, k, xi, wm, wc);
        SS_UNROLL
        for (int i = 0; i < DIN; ++i) {
          R s = m[i];
          SS_UNROLL
          for (int j = 0; j <= i; ++j) s += C[i][j] * xi[j];
          x[i] = s;
        }
        f.eval(x, fx);
        const R sw = ss_sqrt(wc);
        SS_UNROLL
        for (int i = 0; i < DOUT; ++i) {
          const R d = fx[i] - mf[i];
          SS_UNROLL
          for (int j = 0; j < DIN; ++j) S[i][j] += wc * d * xi[j];
          fx[i] = sw * d;
        }
        chol_add_column<R, DOUT>(L, fx);          // L <- tria([L, sqrt(wc) (f_k - m_f)])
      }
    } else {
#pragma unroll 1
      for (int k = 0; k < np; ++k) {
        R xi[DIN], x[DIN], fx[DOUT], wm, wc;
        sigma_point<R, DIN, METHOD>(ru, k, xi, wm, wc);
        SS_UNROLL
        for (int i = 0; i < DIN; ++i) {
          R s = m[i];
          SS_UNROLL
          for (int j = 0; j <= i; ++j) s += C[i][j] * xi[j];
          x[i] = s;
        }
        f.eval(x, fx);
        SS_UNROLL
        for (int i = 0; i < DOUT; ++i) {
          const R d = fx[i] - mf[i];
          SS_UNROLL
          for (int j = 0; j < DIN; ++j) S[i][j] += wc * d * xi[j];
        }
      }
    }
    // F^T = C^{-T} S^T
    R Ft[DIN][DOUT];
    SS_UNROLL
    for (int i = 0; i < DIN; ++i) {
      SS_UNROLL
      for (int j = 0; j < DOUT; ++j) Ft[i][j] = S[j][i];
    }
    solve_lower_T<R, DIN, DOUT>(C, Ft);
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) {
      SS_UNROLL
      for (int j = 0; j < DIN; ++j) F[i][j] = Ft[j][i];
    }
    if (residual) {
#pragma unroll 1
      for (int k = 0; k < np; ++k) {
        R xi[DIN], x[DIN], fx[DOUT], wm, wc;
        sigma_point<R, DIN, METHOD>(ru, k, xi, wm, wc);
        SS_UNROLL
        for (int i = 0; i < DIN; ++i) {
          R s = m[i];
          SS_UNROLL
          for (int j = 0; j <= i; ++j) s += C[i][j] * xi[j];
          x[i] = s;
        }
        f.eval(x, fx);
        const R sw = ss_sqrt(wc);
        SS_UNROLL
        for (int i = 0; i < DOUT; ++i) {
          R e = fx[i] - mf[i];
          SS_UNROLL
          for (int j = 0; j < DIN; ++j) e -= S[i][j] * xi[j];
          fx[i] = sw * e;
        }
        chol_add_column<R, DOUT>(L, fx);
      }
    }
    constexpr bool COND = IsConditional<Fn>::value;
    if constexpr (COND) {
      // L <- tria([L, sqrt(wc_k) chol(Cov[y | x_k]) for every point])
#pragma unroll 1
      for (int k = 0; k < np; ++k) {
        R xi[DIN], x[DIN], wm, wc, ck[DOUT][DOUT];
        sigma_point<R, DIN, METHOD>(ru, k, xi, wm, wc);
        SS_UNROLL
        for (int i = 0; i < DIN; ++i) {
          R s = m[i];
          SS_UNROLL
          for (int j = 0; j <= i; ++j) s += C[i][j] * xi[j];
          x[i] = s;
        }
        f.cond_chol(x, ck);
        const R sw = ss_sqrt(wc);
        SS_UNROLL
        for (int j = 0; j < DOUT; ++j) {
          R col[DOUT];
          SS_UNROLL
          for (int i = 0; i < DOUT; ++i) col[i] = sw * ck[i][j];
          chol_add_column<R, DOUT>(L, col);
        }
      }
    } else {
      // L <- tria([L, qc])
      SS_UNROLL
      for (int j = 0; j < DOUT; ++j) {
        R col[DOUT];
        SS_UNROLL
        for (int i = 0; i < DOUT; ++i) col[i] = qc[i][j];
        chol_add_column<R, DOUT>(L, col);
      }
    }
    if (!residual) {
      // downdate by the columns of F C (= S)
      SS_UNROLL
      for (int j = 0; j < DIN; ++j) {
        R col[DOUT];
        SS_UNROLL
        for (int i = 0; i < DOUT; ++i) col[i] = S[i][j];
        chol_update<R, DOUT>(L, col, R(-1));
      }
    }
    SS_UNROLL
    for (int i = 0; i < DOUT; ++i) {
      R s = COND ? mf[i] : mf[i] + qm[i];
      SS_UNROLL
      for (int j = 0; j < DIN; ++j) s -= F[i][j] * m[j];
      b[i] = s;
    }
  }
}

}  // namespace ss
