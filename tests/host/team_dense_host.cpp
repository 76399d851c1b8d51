// Host build of the team-generic dense kernels (khp_dense.cuh) for the CPU tests: the same
// source that runs as one CTA per matrix on the GPU, run here by a team of one thread
// (TeamSerial).  Matrices are complex, interleaved (re, im), row-major.
#include <vector>

#include "khp_dense.cuh"

using namespace khp;

namespace {

// log_cap > 0: Z updated through a rotation log of log_cap rotations (flushed by the team when
// full), the sweeps left in it applied to every row of Z afterwards, as the GPU does.
template <typename T>
int geev_host(int n, const T* a, T* w, T* lam, int log_cap = 0, bool unwindowed = false) {
  std::vector<cplx<T>> A(n * n), Z(n * n), v(3 * n), win((KHP_HQR_WIN + 2) * (KHP_HQR_WIN + 2)), rs(KHP_HQR_WIN);
  std::vector<cplx<T>> scratch(gehrd_blocked_scratch(n));
  std::vector<T> rc(KHP_HQR_WIN);
  for (int i = 0; i < n * n; ++i) A[i] = mk(a[2 * i], a[2 * i + 1]);
  TeamSerial t;
  TeamShared sh;
  // the reduction the GPU path takes: blocked from n = 64 on
  if (n >= 64) team_gehrd_blocked(t, A.data(), n, n, Z.data(), n, scratch.data(), &sh);
  else team_gehrd(t, A.data(), n, n, Z.data(), n, v.data(), &sh);
  int st;
  if (unwindowed) {
    st = team_hqr(t, A.data(), n, n, Z.data(), n, &sh);
  } else if (log_cap > 0) {
    const int64_t bytes = hqr_log_rot_offset(n) + (int64_t)log_cap * sizeof(HqrRot<T>);
    std::vector<HqrRot<T>> store((bytes + sizeof(HqrRot<T>) - 1) / sizeof(HqrRot<T>));
    const HqrLog<T> L = hqr_log_view<T>(store.data(), bytes, n);
    st = team_hqr_win(t, A.data(), n, n, Z.data(), n, win.data(), rc.data(), rs.data(), &sh, &L);
    for (int i = 0; i < n; ++i) hqr_roll_row(Z.data() + (int64_t)i * n, L.sweeps, L.rot, L.head[0]);
  } else {
    st = team_hqr_win(t, A.data(), n, n, Z.data(), n, win.data(), rc.data(), rs.data(), &sh);
  }
  team_trevc(t, A.data(), n, n, reinterpret_cast<cplx<T>*>(lam));
  team_backtransform(t, Z.data(), n, A.data(), n, n, reinterpret_cast<cplx<T>*>(w), n);
  return st;
}

}  // namespace

extern "C" {

// Hessenberg reduction in place (a becomes H), Q in z; blocked (panels) or one reflector at a time.
int host_gehrd(int n, double* a, double* z, int blocked) {
  TeamSerial t;
  TeamShared sh;
  if (blocked) {
    std::vector<cplx<double>> scratch(gehrd_blocked_scratch(n));
    team_gehrd_blocked(t, reinterpret_cast<cplx<double>*>(a), n, n, reinterpret_cast<cplx<double>*>(z), n,
                       scratch.data(), &sh);
  } else {
    std::vector<cplx<double>> v(3 * n);
    team_gehrd(t, reinterpret_cast<cplx<double>*>(a), n, n, reinterpret_cast<cplx<double>*>(z), n, v.data(), &sh);
  }
  return 0;
}

// Eigenvalues lam [n] and eigenvectors w [n x n] (columns), FP64 / FP32; returns the QR status.
int host_geev(int n, const double* a, double* w, double* lam) { return geev_host<double>(n, a, w, lam); }
int host_geev_f32(int n, const float* a, float* w, float* lam) { return geev_host<float>(n, a, w, lam); }
// The same by the unwindowed sweep (one rotation at a time over all of H and Z).
int host_geev_unwindowed(int n, const double* a, double* w, double* lam) {
  return geev_host<double>(n, a, w, lam, 0, true);
}
int host_geev_unwindowed_f32(int n, const float* a, float* w, float* lam) {
  return geev_host<float>(n, a, w, lam, 0, true);
}
// The same with Z updated through a rotation log of log_cap rotations.
int host_geev_log(int n, const double* a, double* w, double* lam, int log_cap) {
  return geev_host<double>(n, a, w, lam, log_cap);
}
int host_geev_log_f32(int n, const float* a, float* w, float* lam, int log_cap) {
  return geev_host<float>(n, a, w, lam, log_cap);
}

// Solve A X = B (n x m) by the team LU with partial pivoting; a and b overwritten.
int host_gesv(int n, int m, double* a, double* b) {
  std::vector<int> piv(3 * n);
  TeamSerial t;
  TeamShared sh;
  const int st = team_getrf(t, reinterpret_cast<cplx<double>*>(a), n, n, piv.data(), &sh);
  team_getrs(t, reinterpret_cast<cplx<double>*>(a), n, n, piv.data(), reinterpret_cast<cplx<double>*>(b), m, m);
  return st;
}

}  // extern "C"
