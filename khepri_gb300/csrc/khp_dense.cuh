// Dense complex linear algebra written against the Team abstraction (khp_core.cuh):
// LU with partial pivoting, triangular solves / inverse, Householder Hessenberg reduction,
// single-shift complex QR (Schur form) and eigenvectors of the triangular factor.
//
// One team (one CTA) works on one matrix; matrices are row-major with leading dimension ld.
// These are the numerical building blocks of the per-layer mode solve (eig of P*Q,
// khepri/alternative.py:158-178), of build_scatmat (alternative.py:181-195) and of the
// Redheffer star product (alternative.py:19-30), whose reference implementations call LAPACK
// zgeev / zgesv through numpy.
#pragma once

#include "khp_core.cuh"

namespace khp {

template <typename T> KHP_HD T tmax(T a, T b) { return a > b ? a : b; }

// sum_l conj(x[l]) * y[l * sy] with four independent partial sums (memory-level parallelism).
template <typename T>
KHP_HD cplx<T> dotc4(const cplx<T>* x, const cplx<T>* y, int64_t sy, int m) {
  cplx<T> a0 = mk(T(0)), a1 = mk(T(0)), a2 = mk(T(0)), a3 = mk(T(0));
  int l = 0;
  for (; l + 3 < m; l += 4) {
    a0 += conj_mul(x[l], y[l * sy]);
    a1 += conj_mul(x[l + 1], y[(l + 1) * sy]);
    a2 += conj_mul(x[l + 2], y[(l + 2) * sy]);
    a3 += conj_mul(x[l + 3], y[(l + 3) * sy]);
  }
  for (; l < m; ++l) a0 += conj_mul(x[l], y[l * sy]);
  return (a0 + a1) + (a2 + a3);
}

// sum_l x[l] * y[l * sy] with four independent partial sums.
template <typename T>
KHP_HD cplx<T> dotu4s(const cplx<T>* x, const cplx<T>* y, int64_t sy, int m) {
  cplx<T> a0 = mk(T(0)), a1 = mk(T(0)), a2 = mk(T(0)), a3 = mk(T(0));
  int l = 0;
  for (; l + 3 < m; l += 4) {
    fma_acc(a0, x[l], y[l * sy]);
    fma_acc(a1, x[l + 1], y[(l + 1) * sy]);
    fma_acc(a2, x[l + 2], y[(l + 2) * sy]);
    fma_acc(a3, x[l + 3], y[(l + 3) * sy]);
  }
  for (; l < m; ++l) fma_acc(a0, x[l], y[l * sy]);
  return (a0 + a1) + (a2 + a3);
}

// sum_l x[l] * y[l] (contiguous) with four independent partial sums.
template <typename T>
KHP_HD cplx<T> dotu4(const cplx<T>* x, const cplx<T>* y, int m) {
  cplx<T> a0 = mk(T(0)), a1 = mk(T(0)), a2 = mk(T(0)), a3 = mk(T(0));
  int l = 0;
  for (; l + 3 < m; l += 4) {
    fma_acc(a0, x[l], y[l]);
    fma_acc(a1, x[l + 1], y[l + 1]);
    fma_acc(a2, x[l + 2], y[l + 2]);
    fma_acc(a3, x[l + 3], y[l + 3]);
  }
  for (; l < m; ++l) fma_acc(a0, x[l], y[l]);
  return (a0 + a1) + (a2 + a3);
}
template <typename T> KHP_HD T tmin(T a, T b) { return a < b ? a : b; }

// ------------------------------------------------------------------------------------------
// LU factorisation with partial pivoting (row interchanges applied to whole rows).
// A = P L U in place; piv[k] = row swapped with k at step k.  Returns status bits.
// ------------------------------------------------------------------------------------------
template <class Team, typename T>
KHP_HD int team_getrf(const Team& t, cplx<T>* A, int64_t ld, int n, int* piv, TeamShared* sh) {
  int info = 0;
  for (int k = 0; k < n; ++k) {
    T best = T(-1);
    int bi = k;
    for (int i = k + t.tid(); i < n; i += t.size()) {
      const T v = abs1(A[i * ld + k]);
      if (v > best) { best = v; bi = i; }
    }
    team_argmax(t, best, bi, sh);
    if (t.tid() == 0) piv[k] = bi;
    if (!(best > T(0))) {  // zero (or NaN) column: nothing to eliminate
      if (best == T(0)) info |= KHP_BIT_SINGULAR;
      else info |= KHP_BIT_NONFINITE;
      t.sync();
      continue;
    }
    if (bi != k) {
      for (int j = t.tid(); j < n; j += t.size()) {
        const cplx<T> a = A[k * ld + j];
        A[k * ld + j] = A[bi * ld + j];
        A[bi * ld + j] = a;
      }
    }
    t.sync();
    const cplx<T> pv = A[k * ld + k];
    for (int i = k + 1 + t.tid(); i < n; i += t.size()) A[i * ld + k] = cdiv(A[i * ld + k], pv);
    t.sync();
    const int m = n - k - 1;
    for (int e = t.tid(); e < m * m; e += t.size()) {
      const int i = k + 1 + e / m, j = k + 1 + e % m;
      fms_acc(A[i * ld + j], A[i * ld + k], A[k * ld + j]);
    }
    t.sync();
  }
  return info;
}

// Solve A X = B in place in B (n x m, leading dimension ldb) given team_getrf's factors.
template <class Team, typename T>
KHP_HD void team_getrs(const Team& t, const cplx<T>* A, int64_t lda, int n, const int* piv, cplx<T>* B,
                       int64_t ldb, int m) {
  if (2 * m >= t.size()) {
    // Enough right-hand sides for every thread: each owns whole columns, no barriers needed.
    for (int j = t.tid(); j < m; j += t.size()) {
      for (int k = 0; k < n; ++k) {
        const int p = piv[k];
        if (p != k) {
          const cplx<T> a = B[k * ldb + j];
          B[k * ldb + j] = B[p * ldb + j];
          B[p * ldb + j] = a;
        }
      }
      for (int k = 0; k < n; ++k) {
        const cplx<T> bk = B[k * ldb + j];
        for (int i = k + 1; i < n; ++i) fms_acc(B[i * ldb + j], A[i * lda + k], bk);
      }
      for (int k = n - 1; k >= 0; --k) {
        const cplx<T> bk = cdiv(B[k * ldb + j], A[k * lda + k]);
        B[k * ldb + j] = bk;
        for (int i = 0; i < k; ++i) fms_acc(B[i * ldb + j], A[i * lda + k], bk);
      }
    }
    t.sync();
    return;
  }
  for (int j = t.tid(); j < m; j += t.size()) {
    for (int k = 0; k < n; ++k) {
      const int p = piv[k];
      if (p != k) {
        const cplx<T> a = B[k * ldb + j];
        B[k * ldb + j] = B[p * ldb + j];
        B[p * ldb + j] = a;
      }
    }
  }
  t.sync();
  for (int k = 0; k + 1 < n; ++k) {
    const int rows = n - k - 1;
    for (int e = t.tid(); e < rows * m; e += t.size()) {
      const int i = k + 1 + e / m, j = e % m;
      fms_acc(B[i * ldb + j], A[i * lda + k], B[k * ldb + j]);
    }
    t.sync();
  }
  for (int k = n - 1; k >= 0; --k) {
    for (int j = t.tid(); j < m; j += t.size()) B[k * ldb + j] = cdiv(B[k * ldb + j], A[k * lda + k]);
    t.sync();
    for (int e = t.tid(); e < k * m; e += t.size()) {
      const int i = e / m, j = e % m;
      fms_acc(B[i * ldb + j], A[i * lda + k], B[k * ldb + j]);
    }
    t.sync();
  }
}

// Solve X A = B in place in B (m x n rows, leading dimension ldb) given team_getrf's factors
// of A: L U = Pi A with Pi the recorded row interchanges, so X = ((B U^-1) L^-1) Pi.
// Each thread owns whole rows of B (no barriers).
template <class Team, typename T>
KHP_HD void team_getrs_right(const Team& t, const cplx<T>* A, int64_t lda, int n, const int* piv, cplx<T>* B,
                             int64_t ldb, int m) {
  for (int i = t.tid(); i < m; i += t.size()) {
    cplx<T>* x = B + (int64_t)i * ldb;
    for (int j = 0; j < n; ++j) {  // z U = b
      const cplx<T> acc = x[j] - dotu4s(x, A + j, lda, j);
      x[j] = cdiv(acc, A[(int64_t)j * lda + j]);
    }
    for (int j = n - 2; j >= 0; --j) {  // y L = z (L unit lower)
      x[j] = x[j] - dotu4s(x + j + 1, A + (int64_t)(j + 1) * lda + j, lda, n - j - 1);
    }
    for (int k = n - 1; k >= 0; --k) {  // x = y Pi: undo the interchanges, last first
      const int p = piv[k];
      if (p != k) {
        const cplx<T> a = x[k];
        x[k] = x[p];
        x[p] = a;
      }
    }
  }
  t.sync();
}

template <class Team, typename T>
KHP_HD void team_set_identity(const Team& t, cplx<T>* B, int64_t ld, int n, int m) {
  for (int e = t.tid(); e < n * m; e += t.size()) {
    const int i = e / m, j = e % m;
    B[i * ld + j] = mk(T(i == j ? 1 : 0));
  }
  t.sync();
}

// C = alpha * A B + beta * C  (A: n x k, B: k x m).  Plain reference form; the tiled batched
// kernel in khp_gemm.cu is the fast path.
template <class Team, typename T>
KHP_HD void team_gemm(const Team& t, int n, int m, int k, cplx<T> alpha, const cplx<T>* A, int64_t lda,
                      const cplx<T>* B, int64_t ldb, cplx<T> beta, cplx<T>* C, int64_t ldc) {
  const bool use_beta = !(beta.re == T(0) && beta.im == T(0));
  for (int e = t.tid(); e < n * m; e += t.size()) {
    const int i = e / m, j = e % m;
    cplx<T> acc = mk(T(0));
    for (int l = 0; l < k; ++l) fma_acc(acc, A[i * lda + l], B[l * ldb + j]);
    cplx<T> r = alpha * acc;
    if (use_beta) r += beta * C[i * ldc + j];
    C[i * ldc + j] = r;
  }
  t.sync();
}

// ------------------------------------------------------------------------------------------
// Blocked Hessenberg reduction (same reflectors as team_gehrd, applied in panels of KHP_GEHRD_NB
// columns).  With Q_b = H_0 ... H_{nb-1} = I - V T V^H for the panel's reflectors (V unit lower
// trapezoidal, T upper triangular), the panel is reduced column by column against
// Y = A V T (A: the matrix before the panel):
//   column c_j of A Q_j = A[:, c_j] - Y_j conj(V[c_j, 0:j]),   then Q_j^H from the left;
//   Y[:, j] = tau_j (A v_j - Y_j (V_j^H v_j)),   T[0:j, j] = -tau_j T_j (V_j^H v_j);
// and only then is the rest of the matrix updated, once per panel:
//   A[:, J] -= Y V[J, :]^H (right), A[c0+1:, J] -= V T^H (V^H A[c0+1:, J]) (left),
//   Z[:, c0+1:] -= (Z V T) V^H.
// Each column costs one pass over the matrix (A v_j) instead of three read-write passes over
// the matrix and Z.  The reflectors are stored below the subdiagonal (cleared at the end).
// Scratch S (shared memory, gehrd_blocked_scratch(n) entries): the panel's reflectors V and Y
// (reflector-major, n each), T (NB x NB) and the vectors w, u (NB each); needs n >= NB.
// ------------------------------------------------------------------------------------------
#ifndef KHP_GEHRD_NB
#define KHP_GEHRD_NB 8
#endif
// Complex entries of team_gehrd_blocked's scratch for an n x n matrix.
KHP_HD int64_t gehrd_blocked_scratch(int n) {
  return 2 * (int64_t)KHP_GEHRD_NB * n + (int64_t)KHP_GEHRD_NB * KHP_GEHRD_NB + 2 * KHP_GEHRD_NB;
}


template <class Team, typename T>
KHP_HD void team_gehrd_blocked(const Team& t, cplx<T>* H, int64_t ld, int n, cplx<T>* Z, int64_t ldz, cplx<T>* S,
                               TeamShared* sh) {
  // panel width (the per-thread accumulators of the panel updates stay in registers)
  constexpr int NB = KHP_GEHRD_NB;
  const int lanes = t.size() < 32 ? t.size() : 32;
  const int lane = t.tid() % lanes, warp = t.tid() / lanes, nwarps = t.size() / lanes;
  cplx<T>* Vs = S;                  // Vs[l n + i] = V(i, l)
  cplx<T>* Ys = S + NB * n;         // Ys[l n + i] = Y[i][l]
  cplx<T>* Tm = S + 2 * NB * n;     // Tm[m NB + l] = T[m][l]
  cplx<T>* wv = Tm + NB * NB;       // w[l]
  cplx<T>* uv = wv + NB;            // u[l]
  team_set_identity(t, Z, ldz, n, n);
  for (int c0 = 0; c0 + 2 < n; c0 += NB) {
    const int nb = (n - 2 - c0) < NB ? (n - 2 - c0) : NB;
    // V(i, l) of reflector l (column c0 + l): 0 above row c0 + l + 1, 1 there, the stored
    // reflector below; copied to Vs[l n + i] (shared memory, reflector-major) once it is final
    auto V = [&](int i, int l) -> cplx<T> { return Vs[(int64_t)l * n + i]; };
    for (int j = 0; j < nb; ++j) {
      const int c = c0 + j;
      if (j > 0) {
        // column c of A Q_j: b = A[:, c] - Y_j conj(V[c, 0:j]) (every row)
        for (int i = t.tid(); i < n; i += t.size()) {
          cplx<T> acc = H[(int64_t)i * ld + c];
          for (int l = 0; l < j; ++l) acc -= mul_conj(Ys[(int64_t)l * n + i], V(c, l));
          H[(int64_t)i * ld + c] = acc;
        }
        t.sync();
        // w = V_j^H b (rows c0+1..), then w = T_j^H w, then b -= V_j w
        for (int l = warp; l < j; l += nwarps) {
          cplx<T> acc = mk(T(0));
          for (int i = c0 + 1 + lane; i < n; i += lanes) acc += conj_mul(V(i, l), H[(int64_t)i * ld + c]);
          acc = warp_sum(t, acc);
          if (lane == 0) wv[l] = acc;
        }
        t.sync();
        if (t.tid() == 0) {
          for (int l = j - 1; l >= 0; --l) {  // in place, highest first: (T^H w)_l = sum_{m<=l} conj(T_ml) w_m
            cplx<T> acc = mk(T(0));
            for (int m = 0; m <= l; ++m) acc += conj_mul(Tm[m * NB + l], wv[m]);
            wv[l] = acc;
          }
        }
        t.sync();
        for (int i = c0 + 1 + t.tid(); i < n; i += t.size()) {
          cplx<T> acc = H[(int64_t)i * ld + c];
          for (int l = 0; l < j; ++l) acc -= V(i, l) * wv[l];
          H[(int64_t)i * ld + c] = acc;
        }
        t.sync();
      }
      // reflector of column c (rows c+1..)
      T s = T(0);
      for (int i = c + 2 + t.tid(); i < n; i += t.size()) s += norm2(H[(int64_t)i * ld + c]);
      s = team_sum(t, s, sh);
      const cplx<T> alpha = H[(int64_t)(c + 1) * ld + c];
      cplx<T> tau = mk(T(0));
      if (!(s == T(0) && alpha.im == T(0))) {
        const T beta = -copysign(sqrt(norm2(alpha) + s), alpha.re);
        tau = mk((beta - alpha.re) / beta, -alpha.im / beta);
        const cplx<T> scal = cdiv(mk(T(1)), alpha - mk(beta));
        t.sync();  // every thread has read alpha
        for (int i = c + 2 + t.tid(); i < n; i += t.size()) H[(int64_t)i * ld + c] = H[(int64_t)i * ld + c] * scal;
        if (t.tid() == 0) H[(int64_t)(c + 1) * ld + c] = mk(beta);
      }
      t.sync();
      for (int i = t.tid(); i < n; i += t.size())
        Vs[(int64_t)j * n + i] = i <= c ? mk(T(0)) : (i == c + 1 ? mk(T(1)) : H[(int64_t)i * ld + c]);
      t.sync();
      // Y[:, j] = tau (A v - Y_j u), u = V_j^H v;  v = V(., j), A = columns c+1.. of H
      for (int i = t.tid(); i < n; i += t.size()) {
        const cplx<T>* row = H + (int64_t)i * ld;
        cplx<T> acc = row[c + 1];
        for (int col = c + 2; col < n; ++col) fma_acc(acc, row[col], Vs[(int64_t)j * n + col]);
        Ys[(int64_t)j * n + i] = acc;
      }
      for (int l = warp; l < j; l += nwarps) {
        cplx<T> acc = mk(T(0));
        for (int i = c + 1 + lane; i < n; i += lanes) acc += conj_mul(V(i, l), V(i, j));
        acc = warp_sum(t, acc);
        if (lane == 0) uv[l] = acc;
      }
      t.sync();
      for (int i = t.tid(); i < n; i += t.size()) {
        cplx<T> acc = Ys[(int64_t)j * n + i];
        for (int l = 0; l < j; ++l) acc -= Ys[(int64_t)l * n + i] * uv[l];
        Ys[(int64_t)j * n + i] = tau * acc;
      }
      if (t.tid() == 0) {  // T[0:j, j] = -tau T_j u ; T[j][j] = tau
        for (int m = 0; m < j; ++m) {
          cplx<T> acc = mk(T(0));
          for (int l = m; l < j; ++l) fma_acc(acc, Tm[m * NB + l], uv[l]);
          Tm[m * NB + j] = -(tau * acc);
        }
        Tm[j * NB + j] = tau;
        for (int m = j + 1; m < NB; ++m) Tm[m * NB + j] = mk(T(0));
      }
      t.sync();
    }
    const int J0 = c0 + nb;
    // right: A[:, J] -= Y V[J, :]^H for the columns after the panel
    if (J0 < n) {
      // a warp per row (Y's row broadcast), lanes along the row; the loads of PF elements are
      // issued before their stores (the stores would otherwise order every later load)
      constexpr int PF = 4;
      for (int i = warp; i < n; i += nwarps) {
        cplx<T> y[NB];
#pragma unroll
        for (int l = 0; l < NB; ++l) y[l] = l < nb ? Ys[(int64_t)l * n + i] : mk(T(0));
        cplx<T>* hr = H + (int64_t)i * ld;
        for (int J = J0 + lane; J < n; J += PF * lanes) {
          cplx<T> a[PF];
#pragma unroll
          for (int u = 0; u < PF; ++u) a[u] = J + u * lanes < n ? hr[J + u * lanes] : mk(T(0));
#pragma unroll
          for (int u = 0; u < PF; ++u) {
            const int Ju = J + u * lanes;
            if (Ju < n) {
              cplx<T> acc = a[u];
#pragma unroll
              for (int l = 0; l < NB; ++l)
                if (l < nb) acc -= mul_conj(y[l], V(Ju, l));
              hr[Ju] = acc;
            }
          }
        }
      }
      t.sync();
      // left: A[c0+1:, J] -= V T^H (V^H A[c0+1:, J]), thread per column
      for (int J = J0 + t.tid(); J < n; J += t.size()) {
        cplx<T> x[NB];
#pragma unroll
        for (int l = 0; l < NB; ++l) x[l] = mk(T(0));
        for (int i = c0 + 1; i < n; ++i) {
          const cplx<T> a = H[(int64_t)i * ld + J];
#pragma unroll
          for (int l = 0; l < NB; ++l)
            if (l < nb) x[l] += conj_mul(V(i, l), a);
        }
#pragma unroll
        for (int l = NB - 1; l >= 0; --l) {
          if (l >= nb) continue;
          cplx<T> acc = mk(T(0));
#pragma unroll
          for (int q = 0; q < NB; ++q)
            if (q <= l) acc += conj_mul(Tm[q * NB + l], x[q]);
          x[l] = acc;
        }
        for (int i0 = c0 + 1; i0 < n; i0 += PF) {
          cplx<T> a[PF];
#pragma unroll
          for (int u = 0; u < PF; ++u) a[u] = i0 + u < n ? H[(int64_t)(i0 + u) * ld + J] : mk(T(0));
#pragma unroll
          for (int u = 0; u < PF; ++u) {
            if (i0 + u < n) {
              cplx<T> acc = a[u];
#pragma unroll
              for (int l = 0; l < NB; ++l)
                if (l < nb) acc -= V(i0 + u, l) * x[l];
              H[(int64_t)(i0 + u) * ld + J] = acc;
            }
          }
        }
      }
    }
    // Z[:, c0+1:] -= (Z V T) V^H, thread per row of Z
    for (int i = t.tid(); i < n; i += t.size()) {
      cplx<T>* zr = Z + (int64_t)i * ldz;
      cplx<T> x[NB];
#pragma unroll
      for (int l = 0; l < NB; ++l) x[l] = mk(T(0));
      for (int col = c0 + 1; col < n; ++col) {
        const cplx<T> z = zr[col];
#pragma unroll
        for (int l = 0; l < NB; ++l)
          if (l < nb) fma_acc(x[l], z, V(col, l));
      }
#pragma unroll
      for (int l = NB - 1; l >= 0; --l) {  // x <- x T (upper triangular), highest first
        if (l >= nb) continue;
        cplx<T> acc = mk(T(0));
#pragma unroll
        for (int q = 0; q < NB; ++q)
          if (q <= l) fma_acc(acc, x[q], Tm[q * NB + l]);
        x[l] = acc;
      }
      for (int col0 = c0 + 1; col0 < n; col0 += 4) {
        cplx<T> a[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) a[u] = col0 + u < n ? zr[col0 + u] : mk(T(0));
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          if (col0 + u < n) {
            cplx<T> acc = a[u];
#pragma unroll
            for (int l = 0; l < NB; ++l)
              if (l < nb) acc -= mul_conj(x[l], V(col0 + u, l));
            zr[col0 + u] = acc;
          }
        }
      }
    }
    t.sync();
  }
  // clear the reflector storage below the subdiagonal
  for (int e = t.tid(); e < n * n; e += t.size()) {
    const int i = e / n, j = e % n;
    if (i > j + 1) H[(int64_t)i * ld + j] = mk(T(0));
  }
  t.sync();
}

// ------------------------------------------------------------------------------------------
// Hessenberg reduction by Householder reflectors, H = Q^H A Q, Q accumulated into Z.
// Reflector convention: P = I - tau u u^H with u = [1, v], beta real, P^H [alpha; x] = [beta; 0].
// vbuf: n complex of scratch.
// ------------------------------------------------------------------------------------------
template <class Team, typename T>
KHP_HD void team_gehrd(const Team& t, cplx<T>* H, int64_t ld, int n, cplx<T>* Z, int64_t ldz, cplx<T>* vbuf,
                       TeamShared* sh) {
  team_set_identity(t, Z, ldz, n, n);
  for (int k = 0; k + 2 < n; ++k) {
    const int m = n - k - 1;
    T s = T(0);
    for (int i = k + 2 + t.tid(); i < n; i += t.size()) s += norm2(H[i * ld + k]);
    s = team_sum(t, s, sh);
    const cplx<T> alpha = H[(k + 1) * ld + k];
    if (s == T(0) && alpha.im == T(0)) continue;  // already reduced (tau = 0)
    const T beta = -copysign(sqrt(norm2(alpha) + s), alpha.re);
    const cplx<T> tau = mk((beta - alpha.re) / beta, -alpha.im / beta);
    const cplx<T> scal = cdiv(mk(T(1)), alpha - mk(beta));
    for (int l = t.tid(); l < m; l += t.size()) vbuf[l] = (l == 0) ? mk(T(1)) : H[(k + 1 + l) * ld + k] * scal;
    t.sync();
    for (int l = t.tid(); l < m; l += t.size()) H[(k + 1 + l) * ld + k] = (l == 0) ? mk(beta) : mk(T(0));
    // H <- P^H H on rows k+1.., columns k+1..
    const cplx<T> ctau = conj(tau);
    for (int j = k + 1 + t.tid(); j < n; j += t.size()) {
      cplx<T> w = ctau * dotc4(vbuf, H + (int64_t)(k + 1) * ld + j, ld, m);
      for (int l = 0; l < m; ++l) fms_acc(H[(k + 1 + l) * ld + j], vbuf[l], w);
    }
    t.sync();
    // H <- H P on all rows, columns k+1..; Z <- Z P (thread per row: the row is read once for
    // the product and again, from L1, for the update)
    for (int i = t.tid(); i < n; i += t.size()) {
      const cplx<T> y = tau * dotu4(H + (int64_t)i * ld + k + 1, vbuf, m);
      for (int l = 0; l < m; ++l) H[i * ld + k + 1 + l] -= mul_conj(y, vbuf[l]);
      const cplx<T> yz = tau * dotu4(Z + (int64_t)i * ldz + k + 1, vbuf, m);
      for (int l = 0; l < m; ++l) Z[i * ldz + k + 1 + l] -= mul_conj(yz, vbuf[l]);
    }
    t.sync();
  }
}

// ------------------------------------------------------------------------------------------
// Complex Schur form of an upper Hessenberg H by single-shift implicit QR (Wilkinson shift,
// exceptional shifts after 10 and 20 stalled iterations, Ahues-Tisseur deflation test).
// Updates H to upper triangular T and Z <- Z Q.  Returns status bits (NOT_CONVERGED when
// the iteration cap 30*n + 60 is reached: every loop in here is bounded).
// ------------------------------------------------------------------------------------------
// FP32 deflation tolerance in units of FP32's ulp (FP64: always 1).  The FP32 eigensolver only
// starts the FP64 refinement, whose quadratic steps absorb the ~3x larger eigenvalue error;
// measured on 242 x 242 P Q matrices: 12 % fewer rotations at 32 ulp.
#ifndef KHP_HQR_DEFL_F32
#define KHP_HQR_DEFL_F32 32
#endif

template <typename T>
KHP_HD bool hqr_negligible(const cplx<T>* H, int64_t ld, int k, int hi, T smlnum) {
  const cplx<T> h = H[k * ld + k - 1];
  const T ah = abs1(h);
  if (ah <= smlnum) return true;
  const T ulp = Eps<T>::ulp * (sizeof(T) == 4 ? T(KHP_HQR_DEFL_F32) : T(1));
  T tst = abs1(H[(k - 1) * ld + k - 1]) + abs1(H[k * ld + k]);
  if (tst == T(0)) {
    if (k - 2 >= 0) tst += fabs(H[(k - 1) * ld + k - 2].re);
    if (k + 1 <= hi) tst += fabs(H[(k + 1) * ld + k].re);
  }
  if (ah > ulp * tst) return false;
  const T hu = abs1(H[(k - 1) * ld + k]);
  const T ab = tmax(ah, hu), ba = tmin(ah, hu);
  const T d1 = abs1(H[k * ld + k]), d2 = abs1(H[(k - 1) * ld + k - 1] - H[k * ld + k]);
  const T aa = tmax(d1, d2), bb = tmin(d1, d2);
  const T s = aa + ab;
  return ba * (ab / s) <= tmax(smlnum, ulp * (bb * (aa / s)));
}

template <typename T>
KHP_HD cplx<T> hqr_shift(const cplx<T>* H, int64_t ld, int lo, int hi, int its) {
  if (its == 10) return H[lo * ld + lo] + mk(T(0.75) * abs1(H[(lo + 1) * ld + lo]));
  if (its == 20) return H[hi * ld + hi] + mk(T(0.75) * abs1(H[hi * ld + hi - 1]));
  const cplx<T> a = H[(hi - 1) * ld + hi - 1], b = H[(hi - 1) * ld + hi];
  const cplx<T> c = H[hi * ld + hi - 1], d = H[hi * ld + hi];
  const cplx<T> p = T(0.5) * (a - d);
  const cplx<T> bc = b * c;
  cplx<T> disc = csqrt(p * p + bc);
  if (p.re * disc.re + p.im * disc.im < T(0)) disc = -disc;
  const cplx<T> den = p + disc;
  if (den.re == T(0) && den.im == T(0)) return d;
  return d - cdiv(bc, den);
}

// Givens rotation G = [[c, s], [-conj(s), c]] (c real) with G [x; y] = [r; 0].
template <typename T>
KHP_HD void givens(cplx<T> x, cplx<T> y, T& c, cplx<T>& s, cplx<T>& r) {
  const T ax = cabs(x), ay = cabs(y);
  if (ay == T(0)) { c = T(1); s = mk(T(0)); r = x; return; }
  if (ax == T(0)) { c = T(0); s = conj(y) * (T(1) / ay); r = mk(ay); return; }
  const T rho = hypot(ax, ay);
  const cplx<T> ph = x * (T(1) / ax);
  c = ax / rho;
  s = ph * conj(y) * (T(1) / rho);
  r = ph * rho;
}

// FP32 form with reciprocal square roots instead of hypot and divisions (the rotation sits on
// the serial chain of the QR sweep): rho^2 = |x|^2 + |y|^2 in FP32 (the matrices here are far
// from the FP32 overflow / underflow range; a |x|^2 or |y|^2 that underflows to 0 is treated as
// an exact zero).  Unitary to FP32 rounding.
KHP_HD float khp_rsqrt(float v) {
#ifdef __CUDA_ARCH__
  return rsqrtf(v);
#else
  return 1.0f / std::sqrt(v);
#endif
}
template <>
KHP_HD void givens<float>(cplx<float> x, cplx<float> y, float& c, cplx<float>& s, cplx<float>& r) {
  const float ax2 = x.re * x.re + x.im * x.im, ay2 = y.re * y.re + y.im * y.im;
  if (ay2 == 0.f) { c = 1.f; s = mk(0.f); r = x; return; }
  if (ax2 == 0.f) {
    const float iy = khp_rsqrt(ay2);
    c = 0.f;
    s = conj(y) * iy;
    r = mk(ay2 * iy);
    return;
  }
  const float t2 = ax2 + ay2;
  const float ir = khp_rsqrt(t2), ia = khp_rsqrt(ax2);
  c = ax2 * ia * ir;                 // |x| / rho
  s = x * conj(y) * (ia * ir);       // (x / |x|) conj(y) / rho
  r = x * (t2 * ir * ia);            // (x / |x|) rho
}

template <class Team, typename T>
KHP_HD int team_hqr(const Team& t, cplx<T>* H, int64_t ld, int n, cplx<T>* Z, int64_t ldz, TeamShared* sh) {
  const T smlnum = Eps<T>::safemin * (T(n) / Eps<T>::ulp);
  const int cap = 30 * n + 60;
  int hi = n - 1, its = 0, total = 0, status = 0;  // used by thread 0 only
  while (true) {
    t.sync();
    if (t.tid() == 0) {
      int action = 2, lo = 0;
      cplx<T> mu = mk(T(0));
      if (hi >= 0) {
        int l = 0;
        for (int k = hi; k >= 1; --k) {
          if (hqr_negligible(H, ld, k, hi, smlnum)) {
            H[k * ld + k - 1] = mk(T(0));
            l = k;
            break;
          }
        }
        if (l == hi) {
          hi -= 1;
          its = 0;
          action = 1;
        } else {
          ++its;
          ++total;
          if (total > cap) {
            status |= KHP_BIT_NOT_CONVERGED;
          } else {
            action = 0;
            lo = l;
            mu = hqr_shift(H, ld, l, hi, its);
          }
        }
      }
      sh->bi[0] = action;
      sh->bi[1] = lo;
      sh->bi[2] = hi;
      sh->bi[3] = status;
      sh->bd[0] = (double)mu.re;
      sh->bd[1] = (double)mu.im;
    }
    t.sync();
    const int action = sh->bi[0];
    if (action == 2) break;
    if (action == 1) continue;
    const int lo = sh->bi[1], ahi = sh->bi[2];
    const cplx<T> mu = mk((T)sh->bd[0], (T)sh->bd[1]);
    for (int k = lo; k < ahi; ++k) {
      if (t.tid() == 0) {
        cplx<T> x, y;
        if (k == lo) {
          x = H[lo * ld + lo] - mu;
          y = H[(lo + 1) * ld + lo];
        } else {
          x = H[k * ld + k - 1];
          y = H[(k + 1) * ld + k - 1];
        }
        T c;
        cplx<T> s, r;
        givens(x, y, c, s, r);
        if (k > lo) {
          H[k * ld + k - 1] = r;
          H[(k + 1) * ld + k - 1] = mk(T(0));
        }
        sh->bd[2] = (double)c;
        sh->bd[3] = (double)s.re;
        sh->bd[4] = (double)s.im;
      }
      t.sync();
      const T c = (T)sh->bd[2];
      const cplx<T> s = mk((T)sh->bd[3], (T)sh->bd[4]);
      const int j0 = (k == lo) ? lo : k;
      for (int j = j0 + t.tid(); j < n; j += t.size()) {
        const cplx<T> h1 = H[k * ld + j], h2 = H[(k + 1) * ld + j];
        H[k * ld + j] = c * h1 + s * h2;
        H[(k + 1) * ld + j] = c * h2 - conj_mul(s, h1);
      }
      t.sync();
      const int i1 = (k + 2 < ahi) ? k + 2 : ahi;
      for (int i = t.tid(); i <= i1; i += t.size()) {
        const cplx<T> g1 = H[i * ld + k], g2 = H[i * ld + k + 1];
        H[i * ld + k] = c * g1 + mul_conj(g2, s);
        H[i * ld + k + 1] = c * g2 - s * g1;
      }
      for (int i = t.tid(); i < n; i += t.size()) {
        const cplx<T> g1 = Z[i * ldz + k], g2 = Z[i * ldz + k + 1];
        Z[i * ldz + k] = c * g1 + mul_conj(g2, s);
        Z[i * ldz + k + 1] = c * g2 - s * g1;
      }
      t.sync();
    }
  }
  return sh->bi[3];
}

// ------------------------------------------------------------------------------------------
// Rotation log of the QR sweeps.  Z does not feed back into the iteration, so its updates can
// wait: each sweep's rotations are appended to a log and applied to Z later, each row of Z
// rolled through all logged sweeps while it sits in fast memory (k_hqr_apply_log), instead of
// streaming all of Z through DRAM once per sweep.  Every element of Z still receives the same
// rotations in the same order.
//
// Layout of one matrix's log (hqr_log_view): a header of two ints (sweeps, rotations logged,
// written when the QR ends), the (lo, hi) of every sweep (room for the iteration cap's number of
// sweeps), then the rotations of all sweeps in order, sweep s holding the hi - lo rotations
// k = lo .. hi - 1.  When a sweep does not fit in the rotations left, the team applies the log so
// far to Z itself (hqr_log_flush) and starts the log again.
// ------------------------------------------------------------------------------------------
template <typename T>
struct alignas(4 * sizeof(T)) HqrRot {
  T c, sre, sim, pad;  // G = [[c, s], [-conj(s), c]], s = sre + i sim
};

template <typename T>
struct HqrLog {
  int* head;        // [0] sweeps, [1] rotations in the log
  int* sweeps;      // 2 per sweep: lo, hi
  HqrRot<T>* rot;   // rotations in order of application
  int cap_rot;      // rotations the log holds
};

// Upper bound on the sweeps team_hqr_win makes on an n x n matrix (its iteration cap).
KHP_HD int hqr_max_sweeps(int n) { return 30 * n + 61; }

KHP_HD int64_t hqr_log_rot_offset(int n) { return (8 + 8 * (int64_t)hqr_max_sweeps(n) + 31) / 32 * 32; }

// View of a matrix's log in `bytes` bytes at base (32-byte aligned).  cap_rot < n - 1 means the
// region cannot hold one full sweep: the caller then updates Z eagerly.
template <typename T>
KHP_HD HqrLog<T> hqr_log_view(void* base, int64_t bytes, int n) {
  char* p = static_cast<char*>(base);
  HqrLog<T> L;
  L.head = reinterpret_cast<int*>(p);
  L.sweeps = reinterpret_cast<int*>(p + 8);
  const int64_t off = hqr_log_rot_offset(n);
  L.rot = reinterpret_cast<HqrRot<T>*>(p + off);
  const int64_t cap = bytes > off ? (bytes - off) / (int64_t)sizeof(HqrRot<T>) : 0;
  L.cap_rot = cap > 0x3fffffff ? 0x3fffffff : (int)cap;
  return L;
}

// One row of Z through logged sweeps (right rotations, the arithmetic of the eager update).
template <typename T>
KHP_HD void hqr_roll_row(cplx<T>* row, const int* sweeps, const HqrRot<T>* rot, int nsw) {
  int q = 0;
  for (int sw = 0; sw < nsw; ++sw) {
    const int lo = sweeps[2 * sw], hi = sweeps[2 * sw + 1];
    cplx<T> a = row[lo];
    for (int k = lo; k < hi; ++k, ++q) {
      const HqrRot<T> g = rot[q];
      const T c = g.c;
      const cplx<T> s = mk(g.sre, g.sim);
      const cplx<T> b = row[k + 1];
      row[k] = c * a + mul_conj(b, s);
      a = c * b - s * a;
    }
    row[hi] = a;
  }
}

// The team applies the first nsw logged sweeps to Z (thread per row, in place).
template <class Team, typename T>
KHP_HD void hqr_log_flush(const Team& t, const HqrLog<T>& log, int nsw, cplx<T>* Z, int64_t ldz, int n) {
  t.sync();  // the log entries written by every thread are visible
  for (int i = t.tid(); i < n; i += t.size()) hqr_roll_row(Z + (int64_t)i * ldz, log.sweeps, log.rot, nsw);
  t.sync();
}

// Windowed form of the same single-shift QR sweep.  The bulge is chased through a window of
// at most KHP_HQR_WIN rotations held in shared memory (win: (KHP_HQR_WIN + 2)^2 complex), the
// rotations are recorded (rc, rs), and only then applied to the parts of H and Z outside the
// window in one rolling pass per row or column (two live values per thread).  Same rotations,
// same order of application per element as team_hqr; per-step work touches shared memory only.
// With a log, Z is left alone and the rotations go to log->rot from index qbase (the sweep's
// first rotation) on.
#ifndef KHP_HQR_WIN
#define KHP_HQR_WIN 32
#endif

template <class Team, typename T>
KHP_HD void hqr_window_sweep(const Team& t, cplx<T>* H, int64_t ld, int n, cplx<T>* Z, int64_t ldz, int lo, int hi,
                             cplx<T> mu, cplx<T>* win, T* rc, cplx<T>* rs, TeamShared* sh,
                             const HqrLog<T>* log = nullptr, int qbase = 0) {
  constexpr int WS = KHP_HQR_WIN + 2;
  int k0 = lo;
  while (k0 < hi) {
    const int k1 = (k0 + KHP_HQR_WIN - 1 < hi) ? k0 + KHP_HQR_WIN - 1 : hi;
    const int r0 = k0, r1 = (k1 + 1 < hi) ? k1 + 1 : hi;
    const int c0 = (k0 > lo) ? k0 - 1 : k0;
    const int nr = r1 - r0 + 1, nc = k1 - c0 + 1;
    for (int e = t.tid(); e < nr * nc; e += t.size()) {
      const int i = e / nc, j = e % nc;
      win[i * WS + j] = H[(int64_t)(r0 + i) * ld + c0 + j];
    }
    t.sync();
    // The chase touches only the window: warp 0 runs it with warp barriers between steps.
    if (t.tid() < 32) {
      const int lane = t.tid();
      const int lanes = t.size() < 32 ? t.size() : 32;
      for (int k = k0; k < k1; ++k) {
        const int lk = k - r0;  // window row of k
        const int ck = k - c0;  // window column of k
        // every lane forms the same rotation from the same (broadcast) window entries, so c and
        // s come from registers instead of through shared memory from one lane; lane 0 records
        // them for the strip updates and writes r, 0 into column k - 1
        cplx<T> x, y;
        if (k == lo) {
          x = win[lk * WS + ck] - mu;
          y = win[(lk + 1) * WS + ck];
        } else {
          x = win[lk * WS + ck - 1];
          y = win[(lk + 1) * WS + ck - 1];
        }
        T c;
        cplx<T> s, r;
        givens(x, y, c, s, r);
        t.warp_sync();  // every lane has read x and y before the window changes
        if (lane == 0) {
          rc[k - k0] = c;
          rs[k - k0] = s;
          if (k > lo) {
            win[lk * WS + ck - 1] = r;
            win[(lk + 1) * WS + ck - 1] = mk(T(0));
          }
        }
        // row rotation from column k (column k - 1, written above, is not read by the rotations)
        for (int j = ck + lane; j < nc; j += lanes) {
          const cplx<T> h1 = win[lk * WS + j], h2 = win[(lk + 1) * WS + j];
          win[lk * WS + j] = c * h1 + s * h2;
          win[(lk + 1) * WS + j] = c * h2 - conj_mul(s, h1);
        }
        t.warp_sync();
        const int ilast = ((k + 2 < hi) ? k + 2 : hi) - r0;
        for (int i = lane; i <= ilast; i += lanes) {
          const cplx<T> g1 = win[i * WS + ck], g2 = win[i * WS + ck + 1];
          win[i * WS + ck] = c * g1 + mul_conj(g2, s);
          win[i * WS + ck + 1] = c * g2 - s * g1;
        }
        t.warp_sync();
      }
    }
    t.sync();
    for (int e = t.tid(); e < nr * nc; e += t.size()) {
      const int i = e / nc, j = e % nc;
      H[(int64_t)(r0 + i) * ld + c0 + j] = win[i * WS + j];
    }
    const int nrot = k1 - k0;
    if (log) {
      for (int u = t.tid(); u < nrot; u += t.size()) {
        HqrRot<T> g;
        g.c = rc[u];
        g.sre = rs[u].re;
        g.sim = rs[u].im;
        g.pad = T(0);
        log->rot[qbase + (k0 - lo) + u] = g;
      }
    }
    // Each thread's strip is rotated in chunks of RB elements: the chunk's loads are issued
    // together (one memory latency per chunk instead of one per rotation), the running element
    // `a` is carried from chunk to chunk.
    constexpr int RB = 8;
    // rows k0..k1, columns right of the window: left rotations, rolling down the column
    for (int j = k1 + 1 + t.tid(); j < n; j += t.size()) {
      cplx<T> a = H[(int64_t)k0 * ld + j];
      for (int q0 = 0; q0 < nrot; q0 += RB) {
        cplx<T> v[RB];
#pragma unroll
        for (int u = 0; u < RB; ++u)
          if (q0 + u < nrot) v[u] = H[(int64_t)(k0 + q0 + u + 1) * ld + j];
#pragma unroll
        for (int u = 0; u < RB; ++u) {
          if (q0 + u < nrot) {
            const T c = rc[q0 + u];
            const cplx<T> s = rs[q0 + u];
            const cplx<T> b = v[u];
            v[u] = c * a + s * b;  // new value of row k0 + q0 + u
            a = c * b - conj_mul(s, a);
          }
        }
#pragma unroll
        for (int u = 0; u < RB; ++u)
          if (q0 + u < nrot) H[(int64_t)(k0 + q0 + u) * ld + j] = v[u];
      }
      H[(int64_t)k1 * ld + j] = a;
    }
    // rows above the window (columns k0..k1) and every row of Z (unless logged): right
    // rotations, rolling along the row
    const int rows_end = log ? r0 : r0 + n;
    for (int i = t.tid(); i < rows_end; i += t.size()) {
      cplx<T>* row = (i < r0) ? H + (int64_t)i * ld : Z + (int64_t)(i - r0) * ldz;
      cplx<T> a = row[k0];
      for (int q0 = 0; q0 < nrot; q0 += RB) {
        cplx<T> v[RB];
#pragma unroll
        for (int u = 0; u < RB; ++u)
          if (q0 + u < nrot) v[u] = row[k0 + q0 + u + 1];
#pragma unroll
        for (int u = 0; u < RB; ++u) {
          if (q0 + u < nrot) {
            const T c = rc[q0 + u];
            const cplx<T> s = rs[q0 + u];
            const cplx<T> b = v[u];
            v[u] = c * a + mul_conj(b, s);  // new value of column k0 + q0 + u
            a = c * b - s * a;
          }
        }
#pragma unroll
        for (int u = 0; u < RB; ++u)
          if (q0 + u < nrot) row[k0 + q0 + u] = v[u];
      }
      row[k1] = a;
    }
    t.sync();
    k0 = k1;
  }
}

// With a log (log != nullptr, log->cap_rot >= n - 1) Z is updated through the log: the sweeps
// still in the log when the QR ends are left for the caller to apply (hqr_roll_row on every row
// of Z, k_hqr_apply_log on the GPU), their counts in log->head.
template <class Team, typename T>
KHP_HD int team_hqr_win(const Team& t, cplx<T>* H, int64_t ld, int n, cplx<T>* Z, int64_t ldz, cplx<T>* win, T* rc,
                        cplx<T>* rs, TeamShared* sh, const HqrLog<T>* log = nullptr) {
  const T smlnum = Eps<T>::safemin * (T(n) / Eps<T>::ulp);
  const int cap = 30 * n + 60;
  int its = 0, total = 0;  // iteration counters, thread 0 only
  if (t.tid() == 0) {
    sh->bi[2] = n - 1;  // hi
    sh->bi[3] = 0;      // status
    sh->bi[4] = 0;      // sweeps done (diagnostic)
    sh->bi[5] = 0;      // rotations done (diagnostic)
    sh->bi[6] = 0;      // log: flush before this sweep
    sh->bi[7] = 0;      // log: sweeps in the log
    sh->bi[8] = 0;      // log: rotations in the log
    sh->bi[9] = 0;      // log: index of this sweep's first rotation
    sh->bi[10] = 0;     // log: sweeps to apply at a flush
  }
  t.sync();
  while (true) {
    const int hi = sh->bi[2];
    if (hi < 0) break;
    // Largest k in [1, hi] with a negligible subdiagonal H[k][k-1], searched by the whole team.
    T best = T(-1);
    int bk = 0;
    for (int k = 1 + t.tid(); k <= hi; k += t.size()) {
      if (T(k) > best && hqr_negligible(H, ld, k, hi, smlnum)) {
        best = T(k);
        bk = k;
      }
    }
    team_argmax(t, best, bk, sh);
    const int l = best > T(0) ? bk : 0;
    if (t.tid() == 0) {
      if (l > 0) H[(int64_t)l * ld + l - 1] = mk(T(0));
      if (l == hi) {
        sh->bi[2] = hi - 1;
        its = 0;
        sh->bi[0] = 1;
      } else {
        ++its;
        ++total;
        if (total > cap) {
          sh->bi[3] |= KHP_BIT_NOT_CONVERGED;
          sh->bi[2] = -1;
          sh->bi[0] = 2;
        } else {
          const cplx<T> mu = hqr_shift(H, ld, l, hi, its);
          sh->bi[4] += 1;
          sh->bi[5] += hi - l;
          sh->bi[0] = 0;
          sh->bi[1] = l;
          sh->bd[0] = (double)mu.re;
          sh->bd[1] = (double)mu.im;
          if (log) {
            if (sh->bi[8] + (hi - l) > log->cap_rot) {
              // no room for this sweep's hi - l rotations: the team applies the bi[7] sweeps
              // logged so far, then this sweep starts a new log (recorded after the flush)
              sh->bi[6] = 1;
              sh->bi[10] = sh->bi[7];
              sh->bi[7] = 1;
              sh->bi[8] = 0;
            } else {
              sh->bi[6] = 0;
              log->sweeps[2 * sh->bi[7]] = l;
              log->sweeps[2 * sh->bi[7] + 1] = hi;
              sh->bi[7] += 1;
            }
            sh->bi[9] = sh->bi[8];
            sh->bi[8] += hi - l;
          }
        }
      }
    }
    t.sync();
    if (sh->bi[0] != 0) continue;
    const int lo = sh->bi[1];
    if (log && sh->bi[6]) {
      hqr_log_flush(t, *log, sh->bi[10], Z, ldz, n);  // ends with a team barrier
      if (t.tid() == 0) {
        log->sweeps[0] = lo;
        log->sweeps[1] = hi;
      }
    }
    hqr_window_sweep(t, H, ld, n, Z, ldz, lo, hi, mk((T)sh->bd[0], (T)sh->bd[1]), win, rc, rs, sh, log,
                     log ? sh->bi[9] : 0);
  }
  if (log && t.tid() == 0) {
    log->head[0] = sh->bi[7];
    log->head[1] = sh->bi[8];
  }
  t.sync();
  return sh->bi[3];
}

// ------------------------------------------------------------------------------------------
// Eigenvectors of an upper triangular T (in place): lam[k] = T[k][k]; the strictly upper part
// becomes X with T X = X diag(lam), X unit upper triangular.  All eigenvectors are built at
// once, row by row from the bottom; near-equal eigenvalues are separated by a floor
// max(ulp |lam_k|, smlnum) on the divisor.
// ------------------------------------------------------------------------------------------
template <class Team, typename T>
KHP_HD void team_trevc(const Team& t, cplx<T>* H, int64_t ld, int n, cplx<T>* lam) {
  const T smlnum = Eps<T>::safemin * (T(n) / Eps<T>::ulp);
  for (int k = t.tid(); k < n; k += t.size()) lam[k] = H[k * ld + k];
  t.sync();
  for (int e = t.tid(); e < n * n; e += t.size()) {
    const int i = e / n, j = e % n;
    if (i < j) H[i * ld + j] = -H[i * ld + j];
    else H[i * ld + j] = mk(T(i == j ? 1 : 0));
  }
  t.sync();
  for (int j = n - 2; j >= 0; --j) {
    const cplx<T> tjj = lam[j];
    for (int k = j + 1 + t.tid(); k < n; k += t.size()) {
      cplx<T> den = tjj - lam[k];
      const T smin = tmax(Eps<T>::ulp * abs1(lam[k]), smlnum);
      if (abs1(den) < smin) den = mk(smin);
      H[j * ld + k] = cdiv(H[j * ld + k], den);
    }
    t.sync();
    const int cols = n - 1 - j;
    for (int e = t.tid(); e < j * cols; e += t.size()) {
      const int i = e / cols, k = j + 1 + e % cols;
      fma_acc(H[i * ld + k], H[i * ld + j], H[j * ld + k]);
    }
    t.sync();
  }
}

// W = Z X (X unit upper triangular), then every column scaled to unit 2-norm.
template <class Team, typename T>
KHP_HD void team_backtransform(const Team& t, const cplx<T>* Z, int64_t ldz, const cplx<T>* X, int64_t ldx, int n,
                               cplx<T>* W, int64_t ldw) {
  for (int e = t.tid(); e < n * n; e += t.size()) {
    const int i = e / n, k = e % n;
    cplx<T> acc = mk(T(0));
    for (int l = 0; l <= k; ++l) fma_acc(acc, Z[i * ldz + l], X[l * ldx + k]);
    W[i * ldw + k] = acc;
  }
  t.sync();
  for (int k = t.tid(); k < n; k += t.size()) {
    T s = T(0);
    for (int i = 0; i < n; ++i) s += norm2(W[i * ldw + k]);
    const T inv = s > T(0) ? T(1) / sqrt(s) : T(1);
    for (int i = 0; i < n; ++i) W[i * ldw + k] = W[i * ldw + k] * inv;
  }
  t.sync();
}

// Full eigendecomposition A W = W diag(lam).  A is overwritten (Schur factor, then X);
// Z: n x n scratch; vbuf: n scratch; win, rc, rs: window scratch of team_hqr_win.
// Returns status bits.
template <class Team, typename T>
KHP_HD int team_geev(const Team& t, cplx<T>* A, int64_t lda, int n, cplx<T>* Z, int64_t ldz, cplx<T>* W,
                     int64_t ldw, cplx<T>* lam, cplx<T>* vbuf, cplx<T>* win, T* rc, cplx<T>* rs, TeamShared* sh) {
  team_gehrd(t, A, lda, n, Z, ldz, vbuf, sh);
  const int st = team_hqr_win(t, A, lda, n, Z, ldz, win, rc, rs, sh);
  team_trevc(t, A, lda, n, lam);
  team_backtransform(t, Z, ldz, A, lda, n, W, ldw);
  return st;
}

}  // namespace khp
