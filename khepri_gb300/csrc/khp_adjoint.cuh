// Adjoint (reverse-mode) kernels of the mixed-precision stack solve: the transposed interface
// system, its FP32 transposed sweep, the loss seeds from per-order powers and the per-layer
// gradient of a patterned layer's operator M = P Q.  Included by khp_mixed.cu inside its
// anonymous namespace (uses Elem / MapPtrs / Table and the vector helpers defined there).
//
// Notation.  The forward unknowns x (gap amplitudes c+/-, patterned-layer mode amplitudes a+/-,
// r, t) solve F x = b, F being the interface equations evaluated by k_stack_residual.  For a
// real loss L(r, t) with holomorphic partials g = dL/dx, the adjoint y solves F^T y = g and
// every parameter theta of F contributes dL = -2 Re(y^T dF/dtheta x).  A patterned layer enters
// F only through X~ = W diag(exp(-lam k0 d)) W^-1 and Y = V W^-1 (= Q M^-1/2); the gradient with
// respect to M follows from divided differences of f1(mu) = exp(-k0 d sqrt(mu)) and
// f2(mu) = mu^-1/2 (Daleckii-Krein), which stay finite for degenerate eigenvalues.
#pragma once

// y = A^T x for two columns; A row-major n x n, x, y [n][2]; accumulation in A's precision.
template <typename TA, typename TX, typename TY>
__device__ void team_mvT2(const TeamCta& t, const cplx<TA>* A, int n, const cplx<TX>* x, cplx<TY>* y) {
  for (int j = t.tid(); j < n; j += t.size()) {
    cplx<TA> a0 = mk(TA(0)), a1 = mk(TA(0));
    for (int i = 0; i < n; ++i) {
      const cplx<TA> aij = A[(int64_t)i * n + j];
      fma_acc(a0, aij, mk((TA)x[2 * i].re, (TA)x[2 * i].im));
      fma_acc(a1, aij, mk((TA)x[2 * i + 1].re, (TA)x[2 * i + 1].im));
    }
    y[2 * j] = mk((TY)a0.re, (TY)a0.im);
    y[2 * j + 1] = mk((TY)a1.re, (TY)a1.im);
  }
}

// (S_q^T x)_i for a per-harmonic block matrix.
template <typename TX>
__device__ __forceinline__ cd blk_mvT(const M2* S, int q, int nh, int i, int c, const TX* x) {
  const int g = i % nh, rb = i / nh;
  const M2& s = S[g * 4 + q];
  return blk(s, 0, rb) * ld2(x, g, c) + blk(s, 1, rb) * ld2(x, nh + g, c);
}

// (B^T x)_i for one 2x2 block per harmonic (B = V0, V0^-1, ...).
template <typename TX>
__device__ __forceinline__ cd m2T_apply(const M2& m, int rb, int g, int nh, int c, const TX* x) {
  return blk(m, 0, rb) * ld2(x, g, c) + blk(m, 1, rb) * ld2(x, nh + g, c);
}

__device__ __forceinline__ cf to_f(cd z) { return mk((float)z.re, (float)z.im); }

// ------------------------------------------------------------------------------------------
// Loss seeds.  Per-order powers of the reflected and transmitted waves for every polarisation
// (as k_flux_cols; crystal.py:363-396 with only_total=False) and the holomorphic partials of
//   L = sum_{p,g} wR[b][p][g] R_{p,g} + wT[b][p][g] T_{p,g}
// with respect to the two source columns of r and t (GR, GT: [batch][n][2]).  One CTA per
// problem.  wR, wT, Ro, To may be null.
// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_flux_grad(int nh, int npol, const cd* __restrict__ rv,
                                                   const cd* __restrict__ tv, const double* gx, const double* gy,
                                                   const double* kp, const double* k0v, const cd* te_v,
                                                   const cd* tm_v, cd epsi, cd epse, const double* wR,
                                                   const double* wT, double* R, double* Tt, double* Ro, double* To,
                                                   cd* GR, cd* GT) {
  __shared__ TeamShared sh;
  TeamCta t;
  const int64_t b = blockIdx.x;
  const int n = 2 * nh;
  const double k0 = k0v[b];
  const cd kpx = mk(kp[4 * b + 0], kp[4 * b + 1]), kpy = mk(kp[4 * b + 2], kp[4 * b + 3]);
  const cd kzi_abs = conj(csqrt(mk(k0 * k0) * epsi - kpx * kpx - kpy * kpy));
  const cd kzi_n = kzi_abs * (1.0 / k0);
  for (int e = t.tid(); e < 2 * n; e += t.size()) {
    GR[b * 2 * n + e] = mk(0.0);
    GT[b * 2 * n + e] = mk(0.0);
  }
  t.sync();
  for (int pol = 0; pol < npol; ++pol) {
    cd px, py;
    phys::source_pol(kpx, kpy, kzi_abs, te_v[b * npol + pol], tm_v[b * npol + pol], px, py);
    double rs = 0.0, ts = 0.0;
    for (int g = t.tid(); g < nh; g += t.size()) {
      const cd kxa = mk(kp[4 * b + 0] + gx[g], kp[4 * b + 1]);
      const cd kya = mk(kp[4 * b + 2] + gy[g], kp[4 * b + 3]);
      const cd kx = kxa * (1.0 / k0), ky = kya * (1.0 / k0);
      for (int which = 0; which < 2; ++which) {
        const cd* v = (which == 0 ? rv : tv) + b * n * 2;
        const cd eps = which == 0 ? epsi : epse;
        const cd kz = conj(csqrt(mk(k0 * k0) * conj(eps) - kxa * kxa - kya * kya)) * (1.0 / k0);
        const cd sx = v[g * 2 + 0] * px + v[g * 2 + 1] * py;
        const cd sy = v[(nh + g) * 2 + 0] * px + v[(nh + g) * 2 + 1] * py;
        const cd al = -cdiv(kx, kz), be = -cdiv(ky, kz);
        const cd sz = al * sx + be * sy;
        const double cw = kz.re / kzi_n.re;
        const double pg = cw * (norm2(sx) + norm2(sy) + norm2(sz));
        const int64_t o = (b * npol + pol) * nh + g;
        if (which == 0) {
          rs += pg;
          if (Ro) Ro[o] = pg;
        } else {
          ts += pg;
          if (To) To[o] = pg;
        }
        const double* wv = which == 0 ? wR : wT;
        const double w = wv ? wv[o] : 0.0;
        if (w != 0.0) {
          // dP/dsx = cw (conj(sx) + al conj(sz)), dP/dsy = cw (conj(sy) + be conj(sz))
          const cd dx = (conj(sx) + al * conj(sz)) * (w * cw);
          const cd dy = (conj(sy) + be * conj(sz)) * (w * cw);
          cd* G = (which == 0 ? GR : GT) + b * 2 * n;
          G[g * 2 + 0] += dx * px;
          G[g * 2 + 1] += dx * py;
          G[(nh + g) * 2 + 0] += dy * px;
          G[(nh + g) * 2 + 1] += dy * py;
        }
      }
    }
    rs = team_sum(t, rs, &sh);
    ts = team_sum(t, ts, &sh);
    if (threadIdx.x == 0) {
      R[b * npol + pol] = rs;
      Tt[b * npol + pol] = ts;
    }
  }
}

// ------------------------------------------------------------------------------------------
// RHO = F^T y - g in the layout of the unknowns (X, XA, RT), FP64.  Y in the residual layout.
// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_stack_residual_T(Table tb, const double* gx, const double* gy,
                                                          const double* kp, const double* k0v,
                                                          const cd* __restrict__ Y, const cd* __restrict__ GR,
                                                          const cd* __restrict__ GT, cd* RX, cd* RXA, cd* RRT,
                                                          cd* scratch) {
  TeamCta t;
  const int64_t b = blockIdx.x;
  const int nh = tb.nh, n = 2 * nh, L = tb.L;
  const int64_t nn = (int64_t)n * n;
  const int64_t xs = (int64_t)(2 * (L + 1)) * 2 * n, xas = (int64_t)2 * L * 2 * n;
  cd* rx = RX + b * xs;
  cd* rxa = RXA + b * xas;
  cd* rr = RRT + b * 2 * n;
  cd* rt = RRT + (tb.batch + b) * 2 * n;
  const cd* y = Y + b * (int64_t)(L + 2) * 4 * 2 * n;
  cd* p1 = scratch + b * 4 * 2 * n;
  cd* p2 = p1 + 2 * n;
  cd* p3 = p2 + 2 * n;
  cd* p4 = p3 + 2 * n;
  const double k0 = k0v[b];
  auto ys = [&](int elem, int k) { return y + (int64_t)elem * 4 * 2 * n + (int64_t)k * 2 * n; };
  auto cpb = [&](int g) { return rx + (2 * g) * 2 * n; };
  auto cmb = [&](int g) { return rx + (2 * g + 1) * 2 * n; };
  // r, t, and the incidence terms of gap 0
  {
    const M2* S = tb.inc + b * nh * 4;
    const cd* yA = ys(0, 0);
    const cd* yB = ys(0, 1);
    const cd* yBt = ys(L + 1, 1);
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      const int i = e / 2, c = e % 2;
      rr[e] = -yA[e] - GR[b * 2 * n + e];
      rt[e] = -yBt[e] - GT[b * 2 * n + e];
      cpb(0)[e] = -yB[e];
      cmb(0)[e] = blk_mvT(S, 1, nh, i, c, yA) + blk_mvT(S, 3, nh, i, c, yB);
      // every other gap starts from zero
      for (int g = 1; g <= L; ++g) {
        cpb(g)[e] = mk(0.0);
        cmb(g)[e] = mk(0.0);
      }
    }
  }
  t.sync();
  int pl = 0;
  for (int l = 0; l < L; ++l) {
    const Elem& E = tb.e[l];
    const cd* y1 = ys(l + 1, 0);
    const cd* y2 = ys(l + 1, 1);
    cd *cpt = cpb(l), *cmt = cmb(l), *cpd = cpb(l + 1), *cmd = cmb(l + 1);
    if (E.kind == 0) {
      const M2* S = E.blocks + b * nh * 4;
      for (int e = t.tid(); e < 2 * n; e += t.size()) {
        const int i = e / 2, c = e % 2;
        cpt[e] += blk_mvT(S, 0, nh, i, c, y1) + blk_mvT(S, 2, nh, i, c, y2);
        cmt[e] -= y1[e];
        cpd[e] -= y2[e];
        cmd[e] += blk_mvT(S, 1, nh, i, c, y1) + blk_mvT(S, 3, nh, i, c, y2);
      }
      t.sync();
      continue;
    }
    const MapPtrs& M = tb.m[E.slot];
    const cd* W = M.W64 + b * nn;
    const cd* V = M.V64 + b * nn;
    const cd* lam = M.lam64 + b * n;
    const double dk = E.dep.at(b) * k0;
    const cd* y3 = ys(l + 1, 2);
    const cd* y4 = ys(l + 1, 3);
    team_mvT2(t, W, n, y1, p1);
    team_mvT2(t, V, n, y2, p2);
    team_mvT2(t, W, n, y3, p3);
    team_mvT2(t, V, n, y4, p4);
    t.sync();
    cd* rap = rxa + (2 * pl) * 2 * n;
    cd* ram = rxa + (2 * pl + 1) * 2 * n;
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      const int i = e / 2, c = e % 2;
      const int g = i % nh, rb = i / nh;
      const cd xi = xprop(lam, i, dk);
      rap[e] = p1[e] - p2[e] + xi * (p3[e] - p4[e]);
      ram[e] = xi * (p1[e] + p2[e]) + p3[e] + p4[e];
      const M2 v0 = tb.v0b[b * nh + g];
      const cd v2 = m2T_apply(v0, rb, g, nh, c, y2);
      const cd v4 = m2T_apply(v0, rb, g, nh, c, y4);
      cpt[e] += -y1[e] + v2;
      cmt[e] += -y1[e] - v2;
      cpd[e] += -y3[e] + v4;
      cmd[e] += -y3[e] - v4;
    }
    t.sync();
    ++pl;
  }
  {
    const M2* S = tb.trn + b * nh * 4;
    const cd* yA = ys(L + 1, 0);
    const cd* yB = ys(L + 1, 1);
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      const int i = e / 2, c = e % 2;
      cpb(L)[e] += blk_mvT(S, 0, nh, i, c, yA) + blk_mvT(S, 2, nh, i, c, yB);
      cmb(L)[e] -= yA[e];
    }
  }
}

// ------------------------------------------------------------------------------------------
// Transposed FP32 sweep: Y += Sweep^T RHO, Sweep being the linear map of k_stack_sweep
// (residual -> correction).  Statements of k_stack_sweep in reverse order, each transposed.
// Per-problem FP32 workspace [..][n][2]: s-bar at every gap (L+1), per layer 4 vectors, 8 temps.
// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_stack_sweep_T(Table tb, const double* gx, const double* gy,
                                                       const double* kp, const double* k0v, const cd* __restrict__ RX,
                                                       const cd* __restrict__ RXA, const cd* __restrict__ RRT, cd* Y,
                                                       cf* WS) {
  TeamCta t;
  const int64_t b = blockIdx.x;
  const int nh = tb.nh, n = 2 * nh, L = tb.L;
  const int64_t nn = (int64_t)n * n;
  const int64_t xs = (int64_t)(2 * (L + 1)) * 2 * n, xas = (int64_t)2 * L * 2 * n;
  const cd* rx = RX + b * xs;
  const cd* rxa = RXA + b * xas;
  const cd* rr = RRT + b * 2 * n;
  const cd* rt = RRT + (tb.batch + b) * 2 * n;
  cd* y = Y + b * (int64_t)(L + 2) * 4 * 2 * n;
  const int64_t wsz = (int64_t)(L + 1 + 4 * L + 8) * 2 * n;
  cf* ws = WS + b * wsz;
  auto SB = [&](int g) { return ws + (int64_t)g * 2 * n; };
  auto LV = [&](int l, int k) { return ws + (int64_t)(L + 1 + 4 * l + k) * 2 * n; };
  cf* T0 = ws + (int64_t)(L + 1 + 4 * L) * 2 * n;
  cf* T1 = T0 + 2 * n;
  cf* T2 = T1 + 2 * n;
  cf* T3 = T2 + 2 * n;
  cf* dp = T3 + 2 * n;  // running dcp-bar
  cf* T4 = dp + 2 * n;
  cf* T5 = T4 + 2 * n;
  cf* T6 = T5 + 2 * n;
  const double k0 = k0v[b];
  auto ys = [&](int elem, int k) { return y + (int64_t)elem * 4 * 2 * n + (int64_t)k * 2 * n; };
  auto gam = [&](int g) { return tb.gam + ((int64_t)g * tb.batch + b) * nn; };
  auto rcp = [&](int g) { return rx + (2 * g) * 2 * n; };
  auto rcm = [&](int g) { return rx + (2 * g + 1) * 2 * n; };
  for (int g = 0; g <= L; ++g)
    for (int e = t.tid(); e < 2 * n; e += t.size()) SB(g)[e] = mk(0.f);
  // ---- emergence: t = S21 dcp_L + rB ----
  {
    const M2* S = tb.trn + b * nh * 4;
    cd* yB = ys(L + 1, 1);
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      const int i = e / 2, c = e % 2;
      yB[e] += rt[e];
      dp[e] = to_f(blk_mvT(S, 2, nh, i, c, rt));
    }
    t.sync();
  }
  // ---- forward part, reversed ----
  int pl_count = 0;
  for (int l = 0; l < L; ++l) pl_count += tb.e[l].kind == 1;
  int pl = pl_count;
  for (int l = L - 1; l >= 0; --l) {
    const Elem& E = tb.e[l];
    // gap l+1: dcm = Gamma dcp + s ; both recorded
    for (int e = t.tid(); e < 2 * n; e += t.size()) T0[e] = to_f(rcm(l + 1)[e]);  // dcm-bar
    t.sync();
    team_mvT2(t, gam(l + 1), n, T0, T1);
    t.sync();
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      dp[e] = dp[e] + to_f(rcp(l + 1)[e]) + T1[e];
      SB(l + 1)[e] = SB(l + 1)[e] + T0[e];
    }
    t.sync();
    if (E.kind == 0) {
      // dcp_{l+1} = inv1 (S21 dcp_l + w)
      const M2* S = E.blocks + b * nh * 4;
      cf* wb = LV(l, 0);
      team_mvT2(t, E.inv1 + b * nn, n, dp, wb);
      t.sync();
      for (int e = t.tid(); e < 2 * n; e += t.size()) {
        const int i = e / 2, c = e % 2;
        dp[e] = to_f(blk_mvT(S, 2, nh, i, c, wb));
      }
      t.sync();
      continue;
    }
    --pl;
    const MapPtrs& M = tb.m[E.slot];
    const double dk = E.dep.at(b) * k0;
    const cf* lam = M.lam32 + b * n;
    const cd* rap = rxa + (2 * pl) * 2 * n;
    const cd* ram = rxa + (2 * pl + 1) * 2 * n;
    cf* k1b = LV(l, 0);
    cf* k2b = LV(l, 1);
    cf* hb = LV(l, 2);
    cf* qb = LV(l, 3);
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      T0[e] = to_f(ram[e]);  // T3'-bar
      hb[e] = T0[e];
    }
    t.sync();
    team_mvT2(t, E.zr + b * nn, n, T0, T1);    // (X a+)-bar from rho X a+
    team_mvT2(t, E.inv1 + b * nn, n, dp, T2);  // T2-bar
    t.sync();
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      qb[e] = T2[e];
      const cd xbar = ld2(T1, e / 2, e % 2) + 2.0 * ld2(T2, e / 2, e % 2);
      const cd xi = cexp(-(mk((double)lam[e / 2].re, (double)lam[e / 2].im) * dk));
      T3[e] = to_f(rap[e] + xi * xbar);  // a+-bar
    }
    t.sync();
    team_mvT2(t, E.inv2 + b * nn, n, T3, T4);  // T3-bar
    t.sync();
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      dp[e] = mk(2.f, 0.f) * T4[e];
      k1b[e] = mk(0.f) - T4[e];
      k2b[e] = T4[e];
    }
    t.sync();
  }
  // ---- incidence, reversed ----
  {
    const M2* S = tb.inc + b * nh * 4;
    cd* yA = ys(0, 0);
    cd* yB = ys(0, 1);
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      const int i = e / 2, c = e % 2;
      T0[e] = to_f(blk_mvT(S, 1, nh, i, c, rr) + rcm(0)[e]);  // dcm0-bar
      yA[e] += rr[e];
    }
    t.sync();
    team_mvT2(t, gam(0), n, T0, T1);
    t.sync();
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      dp[e] = dp[e] + to_f(rcp(0)[e]) + T1[e];
      SB(0)[e] = SB(0)[e] + T0[e];
    }
    t.sync();
    team_mvT2(t, tb.inv0 + b * nn, n, dp, T2);  // u
    t.sync();
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      const int i = e / 2, c = e % 2;
      SB(0)[e] = SB(0)[e] + to_f(blk_mvT(S, 3, nh, i, c, T2));
      yB[e] += ld2(T2, i, c);
    }
    t.sync();
  }
  // ---- backward part, reversed (gaps 0 .. L-1) ----
  for (int l = 0; l < L; ++l) {
    const Elem& E = tb.e[l];
    cf* sl = SB(l);
    cf* sj = SB(l + 1);
    cd* f1 = ys(l + 1, 0);
    cd* f2 = ys(l + 1, 1);
    if (E.kind == 0) {
      const M2* S = E.blocks + b * nh * 4;
      const cf* wfwd = LV(l, 0);
      for (int e = t.tid(); e < 2 * n; e += t.size()) {
        const int i = e / 2, c = e % 2;
        f1[e] += ld2(sl, i, c);
        T1[e] = to_f(blk_mvT(S, 1, nh, i, c, sl));  // T1-bar
      }
      t.sync();
      team_mvT2(t, E.zr + b * nn, n, T1, T2);  // Z^T T1-bar
      t.sync();
      for (int e = t.tid(); e < 2 * n; e += t.size()) T3[e] = wfwd[e] + T2[e];  // w-bar
      t.sync();
      for (int e = t.tid(); e < 2 * n; e += t.size()) {
        const int i = e / 2, c = e % 2;
        sj[e] = sj[e] + T1[e] + to_f(blk_mvT(S, 3, nh, i, c, T3));
        f2[e] += ld2(T3, i, c);
      }
      t.sync();
      continue;
    }
    const MapPtrs& M = tb.m[E.slot];
    const double dk = E.dep.at(b) * k0;
    const cf* lam = M.lam32 + b * n;
    cd* f3 = ys(l + 1, 2);
    cd* f4 = ys(l + 1, 3);
    cf* k1b = LV(l, 0);
    cf* k2b = LV(l, 1);
    cf* hb = LV(l, 2);
    cf* qb = LV(l, 3);
    for (int e = t.tid(); e < 2 * n; e += t.size()) T0[e] = mk(0.5f, 0.f) * sl[e];
    t.sync();
    team_mvT2(t, gam(l), n, T0, T1);  // T3-bar = 1/2 Gamma^T s-bar
    t.sync();
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      k1b[e] = k1b[e] + T0[e] - T1[e];
      k2b[e] = k2b[e] + T0[e] + T1[e];
    }
    t.sync();  // the V0^-T product below reads other threads' k2b entries
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      const int i = e / 2, c = e % 2;
      const int g = i % nh, rb = i / nh;
      f1[e] += ld2(k1b, i, c);
      const M2 vi = tb.v0ib[b * nh + g];
      const cd z = m2T_apply(vi, rb, g, nh, c, k2b);
      f2[e] += z;
      T2[e] = to_f(z);
    }
    t.sync();
    team_mvT2(t, M.V32 + b * nn, n, T2, T3);  // V^T z
    team_mvT2(t, M.W32 + b * nn, n, k1b, T4);  // W^T k1-bar
    t.sync();
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      const cd xi = cexp(-(mk((double)lam[e / 2].re, (double)lam[e / 2].im) * dk));
      const cd hv = ld2(hb, e / 2, e % 2) + xi * (ld2(T3, e / 2, e % 2) + ld2(T4, e / 2, e % 2));
      hb[e] = to_f(hv);
      T0[e] = mk(0.5f, 0.f) * hb[e];
    }
    t.sync();
    team_mvT2(t, E.zr + b * nn, n, T0, T1);  // 1/2 rho^T h-bar
    t.sync();
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      const cf qv = qb[e] + T1[e];
      T5[e] = qv - T0[e];                 // g3-bar = -1/2 h-bar + q-bar
      T6[e] = mk(0.f) - T0[e] - qv;       // g4-bar = -1/2 h-bar - q-bar
    }
    t.sync();
    team_mvT2(t, M.Wi + b * nn, n, T5, T2);  // T0-bar
    team_mvT2(t, M.Vi + b * nn, n, T6, T3);  // T1-bar
    t.sync();
    for (int e = t.tid(); e < 2 * n; e += t.size()) {
      const int i = e / 2, c = e % 2;
      const int g = i % nh, rb = i / nh;
      f3[e] += ld2(T2, i, c);
      f4[e] += ld2(T3, i, c);
      const M2 v0 = tb.v0b[b * nh + g];
      const cd sv = ld2(sj, i, c) - ld2(T2, i, c) - m2T_apply(v0, rb, g, nh, c, T3);
      sj[e] = to_f(sv);
    }
    t.sync();
  }
  {
    cd* yA = ys(L + 1, 0);
    const cf* sL = SB(L);
    for (int e = t.tid(); e < 2 * n; e += t.size()) yA[e] += ld2(sL, e / 2, e % 2);
  }
}

// ------------------------------------------------------------------------------------------
// Gradient of one patterned layer with respect to its M = P Q and its Q (direct term of
// Y = Q f2(M)), accumulated transposed: HT += (G1 o D1 + G2 o D2)^T, QDT += Qbar_direct^T, with
//   G1 = (W^T y1 + V^T y2) a-^T + (W^T y3 - V^T y4) a+^T,
//   G2 = diag(lam) [(V^T y2) w2^T + (V^T y4) w4^T],   w2 = X a- - a+,  w4 = a- - X a+,
//   Qbar_direct = y2 (W (w2 / lam))^T + y4 (W (w4 / lam))^T,
// summed over the two source columns; D1, D2 the divided differences of f1, f2 at mu = lam^2.
// Step 1 (one CTA per problem): the n-vectors, VEC per problem 10 x [n][2]:
//   u1 = W^T y1 + V^T y2, u3 = W^T y3 - V^T y4, v2 = V^T y2, v4 = V^T y4, w2, w4,
//   s2 = w2 / lam, s4 = w4 / lam, z2 = W s2, z4 = W s4.
// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_layer_vectors(Table tb, int l, int pl, const double* k0v,
                                                       const cd* __restrict__ XA, const cd* __restrict__ Y, cd* VEC) {
  TeamCta t;
  const int64_t b = blockIdx.x;
  const int nh = tb.nh, n = 2 * nh, L = tb.L;
  const int64_t nn = (int64_t)n * n;
  const int64_t xas = (int64_t)2 * L * 2 * n;
  const Elem& E = tb.e[l];
  const MapPtrs& M = tb.m[E.slot];
  const cd* W = M.W64 + b * nn;
  const cd* V = M.V64 + b * nn;
  const cd* lam = M.lam64 + b * n;
  const double dk = E.dep.at(b) * k0v[b];
  const cd* ap = XA + b * xas + (2 * pl) * 2 * n;
  const cd* am = XA + b * xas + (2 * pl + 1) * 2 * n;
  const cd* y = Y + b * (int64_t)(L + 2) * 4 * 2 * n + (int64_t)(l + 1) * 4 * 2 * n;
  const cd *y1 = y, *y2 = y + 2 * n, *y3 = y + 4 * n, *y4 = y + 6 * n;
  cd* v = VEC + b * 20 * n;
  cd *u1 = v, *u3 = v + 2 * n, *v2 = v + 4 * n, *v4 = v + 6 * n, *w2 = v + 8 * n, *w4 = v + 10 * n;
  cd *s2 = v + 12 * n, *s4 = v + 14 * n, *z2 = v + 16 * n, *z4 = v + 18 * n;
  team_mvT2(t, W, n, y1, u1);
  team_mvT2(t, V, n, y2, v2);
  team_mvT2(t, W, n, y3, u3);
  team_mvT2(t, V, n, y4, v4);
  for (int e = t.tid(); e < 2 * n; e += t.size()) {
    const cd xi = xprop(lam, e / 2, dk);
    const cd a = xi * am[e] - ap[e], c = am[e] - xi * ap[e];
    const cd li = cdiv(mk(1.0), lam[e / 2]);
    w2[e] = a;
    w4[e] = c;
    s2[e] = a * li;
    s4[e] = c * li;
  }
  t.sync();
  for (int e = t.tid(); e < 2 * n; e += t.size()) {
    u1[e] += v2[e];
    u3[e] -= v4[e];
  }
  team_mv2(t, W, n, s2, z2);
  team_mv2(t, W, n, s4, z4);
}

// Divided difference (f(mu_i) - f(mu_j)) / (mu_i - mu_j), mu = lam^2, for
// f1 = exp(-tau lam) (kind 1) and f2 = 1 / lam (kind 2); f'(mu) on the diagonal and for
// numerically equal arguments.
__device__ __forceinline__ cd phi_exp(cd z) {
  // (exp(z) - 1) / z
  if (cabs(z) < 1e-4) return mk(1.0) + z * 0.5 + z * z * (1.0 / 6.0);
  return cdiv(cexp(z) - mk(1.0), z);
}
__device__ __forceinline__ cd divdiff_f1(cd li, cd lj, double tau) {
  // (e^{-tau li} - e^{-tau lj}) / ((li - lj)(li + lj)) = -tau e^{-tau lj} phi(-tau (li - lj)) / (li + lj)
  const cd ej = cexp(-(lj * tau));
  return cdiv(-(ej * phi_exp(-((li - lj) * tau))) * tau, li + lj);
}
__device__ __forceinline__ cd divdiff_f2(cd li, cd lj) {
  // (1/li - 1/lj) / ((li - lj)(li + lj)) = -1 / (li lj (li + lj))
  return cdiv(mk(-1.0), li * lj * (li + lj));
}

// Step 2 (element-wise over [batch][n][n]): HT[j][i] += G1_ij D1_ij + G2_ij D2_ij and
// QDT[j][i] += Qbar_direct_ij.
__global__ void k_layer_accum(int64_t batch, int n, const cd* __restrict__ lam64, DepthSel dep, const double* k0v,
                              const cd* __restrict__ XA, int64_t xas, int pl, const cd* __restrict__ Y,
                              int64_t ys_stride, int64_t ys_off, const cd* __restrict__ VEC, cd* HT, cd* QDT) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < batch * nn; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = e / nn;
    const int rc = (int)(e % nn);
    const int i = rc / n, j = rc % n;
    const cd* v = VEC + b * 20 * n;
    const cd *u1 = v, *u3 = v + 2 * n, *v2 = v + 4 * n, *v4 = v + 6 * n, *w2 = v + 8 * n, *w4 = v + 10 * n;
    const cd *z2 = v + 16 * n, *z4 = v + 18 * n;
    const cd* ap = XA + b * xas + (2 * pl) * 2 * n;
    const cd* am = XA + b * xas + (2 * pl + 1) * 2 * n;
    const cd* y = Y + b * ys_stride + ys_off;
    const cd *y2 = y + 2 * n, *y4 = y + 6 * n;
    const cd* lam = lam64 + b * n;
    const double tau = dep.at(b) * k0v[b];
    const cd li = lam[i], lj = lam[j];
    cd g1 = mk(0.0), g2 = mk(0.0), qd = mk(0.0);
    for (int c = 0; c < 2; ++c) {
      g1 += u1[2 * i + c] * am[2 * j + c] + u3[2 * i + c] * ap[2 * j + c];
      g2 += v2[2 * i + c] * w2[2 * j + c] + v4[2 * i + c] * w4[2 * j + c];
      qd += y2[2 * i + c] * z2[2 * j + c] + y4[2 * i + c] * z4[2 * j + c];
    }
    g2 = g2 * li;
    const cd h = g1 * divdiff_f1(li, lj, tau) + g2 * divdiff_f2(li, lj);
    HT[b * nn + (int64_t)j * n + i] += h;
    QDT[b * nn + (int64_t)j * n + i] += qd;
  }
}
