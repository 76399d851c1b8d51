// Per-harmonic physics shared by the batched kernels: normalised k-vectors, the square-root
// branches of the reference, homogeneous-medium Q blocks, free-space V0 blocks and the incident
// polarisation.  All in FP64 (these are O(n) quantities; storage precision is chosen by callers).
#pragma once

#include "khp_core.cuh"

namespace khp {
namespace phys {

using cd = cplx<double>;

// 2x2 complex matrix [[a, b], [c, d]] (one harmonic's block of a "diagonal-block" matrix).
struct M2 {
  cd a, b, c, d;
};
KHP_HD M2 m2(cd a, cd b, cd c, cd d) { return M2{a, b, c, d}; }
KHP_HD M2 mul(const M2& x, const M2& y) {
  return m2(x.a * y.a + x.b * y.c, x.a * y.b + x.b * y.d, x.c * y.a + x.d * y.c, x.c * y.b + x.d * y.d);
}
KHP_HD M2 add(const M2& x, const M2& y) { return m2(x.a + y.a, x.b + y.b, x.c + y.c, x.d + y.d); }
KHP_HD M2 sub(const M2& x, const M2& y) { return m2(x.a - y.a, x.b - y.b, x.c - y.c, x.d - y.d); }
KHP_HD M2 scale(cd s, const M2& x) { return m2(s * x.a, s * x.b, s * x.c, s * x.d); }
KHP_HD M2 eye2() { return m2(mk(1.0), mk(0.0), mk(0.0), mk(1.0)); }
KHP_HD M2 inv2(const M2& x) {
  const cd r = cdiv(mk(1.0), x.a * x.d - x.b * x.c);
  return m2(r * x.d, -(r * x.b), -(r * x.c), r * x.a);
}

// (kp + G_g) / k0 for problem b (khepri/expansion.py:43-50); kp: [batch][2] complex as doubles.
KHP_HD void kvec(const double* kp, const double* k0, const double* gx, const double* gy, int64_t b, int g, cd& kx,
                 cd& ky) {
  const double k = k0[b];
  kx = mk((kp[4 * b + 0] + gx[g]) / k, kp[4 * b + 1] / k);
  ky = mk((kp[4 * b + 2] + gy[g]) / k, kp[4 * b + 3] / k);
}

// Homogeneous-layer / free-space branch: Re(arg) < 0 -> -i sqrt(-arg) (alternative.py:92-96, 145-149).
KHP_HD cd kz_branch(cd arg) {
  if (arg.re < 0.0) {
    const cd r = csqrt(-arg);
    return mk(r.im, -r.re);
  }
  return csqrt(arg);
}

// Q block of a homogeneous medium (alternative.py:36-39, 133-135).
KHP_HD M2 q_medium(cd kx, cd ky, cd eps) {
  const cd kxy = kx * ky;
  return m2(kxy, eps - kx * kx, ky * ky - eps, -kxy);
}

// Free-space V0 block Q0 / (i kz0) (alternative.py:84-99).
KHP_HD M2 v0_block(cd kx, cd ky) {
  const cd one = mk(1.0);
  const cd kz0 = kz_branch(one - kx * kx - ky * ky);
  return scale(cdiv(one, mk(-kz0.im, kz0.re)), q_medium(kx, ky, one));
}

// The four 2x2 blocks (S11, S12, S21, S22) of a homogeneous medium's S-matrix for one harmonic:
// kind 0 uniform layer (alternative.py:130-156 + build_scatmat 181-195), 1 incidence half-space
// (alternative.py:32-56), 2 emergence half-space (alternative.py:59-82).  Also its V block and
// eigenvalue.
KHP_HD void homogeneous_blocks(int kind, cd kx, cd ky, cd eps, double dk0, M2 s[4], M2& vm, cd& lm) {
  const cd one = mk(1.0);
  const M2 v0 = v0_block(kx, ky);
  if (kind == 0) {
    const cd kz = kz_branch(eps - kx * kx - ky * ky);
    lm = mk(-kz.im, kz.re);
    vm = scale(cdiv(one, lm), q_medium(kx, ky, eps));
    const M2 t2 = mul(inv2(vm), v0);
    const M2 A = add(eye2(), t2), B = sub(eye2(), t2);
    const cd x = cexp(-(lm * dk0));
    const cd x2 = x * x;
    const M2 bab = mul(mul(B, inv2(A)), B);
    const M2 tinv = inv2(sub(A, scale(x2, bab)));
    s[0] = scale(x2 - one, mul(tinv, B));
    s[1] = scale(x, mul(tinv, sub(A, bab)));
    s[2] = s[1];
    s[3] = s[0];
    return;
  }
  const cd kz = conj(csqrt(eps - kx * kx - ky * ky));
  lm = mk(-kz.im, kz.re);
  vm = scale(cdiv(one, lm), q_medium(kx, ky, eps));
  const M2 t2 = mul(inv2(v0), vm);
  const M2 A = add(eye2(), t2), B = sub(eye2(), t2);
  const M2 ai = inv2(A);
  const M2 aib = mul(ai, B);
  const M2 half = scale(mk(0.5), sub(A, mul(B, aib)));
  if (kind == 1) {
    s[0] = scale(mk(-1.0), aib);
    s[1] = scale(mk(2.0), ai);
    s[2] = half;
    s[3] = mul(B, ai);
  } else {
    s[0] = mul(B, ai);
    s[1] = half;
    s[2] = scale(mk(2.0), ai);
    s[3] = scale(mk(-1.0), aib);
  }
}

// Polarisation (x, y components) of the incident plane wave, alternative.py:101-128:
// (te, tm) normalised; aTE = -(z_dev x kbar)/|.|, z_dev = (0, 0, -1); aTM = aTE x kbar/|.|;
// at |kp| < 1e-8, aTE = x and aTM = y.  kzi_abs: conj(sqrt(k0^2 epsi - kp^2)).
KHP_HD void source_pol(cd kpx, cd kpy, cd kzi_abs, cd te, cd tm, cd& px, cd& py) {
  const double kpn = sqrt(norm2(kpx) + norm2(kpy));
  const double kn = sqrt(norm2(kpx) + norm2(kpy) + norm2(kzi_abs));
  const double pn = hypot(cabs(te), cabs(tm));
  te = te * (1.0 / pn);
  tm = tm * (1.0 / pn);
  if (fabs(kpn) < 1e-8) {
    px = te;
    py = tm;
    return;
  }
  const cd bx = kpx * (1.0 / kn), by = kpy * (1.0 / kn), bz = kzi_abs * (1.0 / kn);
  cd ex = -by, ey = bx;
  const double ne = sqrt(norm2(ex) + norm2(ey));
  ex = ex * (1.0 / ne);
  ey = ey * (1.0 / ne);
  cd mx = ey * bz, my = -(ex * bz), mz = ex * by - ey * bx;
  const double nm = sqrt(norm2(mx) + norm2(my) + norm2(mz));
  mx = mx * (1.0 / nm);
  my = my * (1.0 / nm);
  px = te * ex + tm * mx;
  py = te * ey + tm * my;
}

}  // namespace phys
}  // namespace khp
