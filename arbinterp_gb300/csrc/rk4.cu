// Particle trajectories through a 3D interpolated field, fused on the device.
//
// The reference was written to simulate particle motion in magnetic fields
// and planned numerical integrators for it (CHANGELOG.md, v1.0.0); its users
// call Query in a Python loop, one round trip per stage.  Here one thread
// carries one particle through every step: classical fourth-order
// Runge-Kutta on
//     x' = v,   v' = coef * grad f(x) + gravity
// with f the interpolated scalar (scalar and norm modes) or |B| (both mode),
// e.g. coef = -mu/m for a weak-field seeker in a magnetic trap.  Each stage
// evaluates the interpolant on the fly (float64 or the float32 mixed path,
// as the interpolant's queries do).  A stage outside the interpolation
// volume, or on a cell index at or past nc (the upper faces), ends the
// particle: its state becomes NaN and it is counted in lost[0].
#include "eval.cuh"

namespace arb {

// Acceleration at x; false when x is outside the interpolation volume.
template <int F, bool MIXED>
__device__ __forceinline__ bool rk4_accel(const arb_grid &g, const KParams &kp, const double x[3], double coef,
                                          const double grav[3], double a[3]) {
  using T = typename std::conditional<MIXED, float, double>::type;
  T fr[3];
  CoordStep s;
  if constexpr (MIXED)
    s = coord_step_fast<3>(x, kp.ax, g, fr);
  else
    s = coord_step<3, true>(x, g, kp.inv_h, fr);
  if (s.oob || s.nan || s.idx >= g.nc) return false;
  int64_t c[3];
  cell_from_step<3>(s, g, c);
  double val[F], grad[3] = {0.0, 0.0, 0.0};
  eval_otf3<F, MIXED>(g, kp, c, fr, val, grad);
#pragma unroll
  for (int a_ = 0; a_ < 3; ++a_) a[a_] = coef * grad[a_] + grav[a_];
  return true;
}

template <int F, bool MIXED>
__global__ void __launch_bounds__(128) rk4_kernel(arb_grid g, KParams kp, double *state, int64_t n, double dt,
                                                  int64_t nsteps, double coef, double g0, double g1, double g2,
                                                  double *path, int64_t rec_every, unsigned long long *lost) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double *st = state + i * 6;
  double x[3] = {st[0], st[1], st[2]}, v[3] = {st[3], st[4], st[5]};
  const double grav[3] = {g0, g1, g2};
  const double h2 = 0.5 * dt, h6 = dt / 6.0;
  bool alive = true;
#pragma unroll
  for (int a = 0; a < 3; ++a) alive &= (x[a] == x[a]) && (v[a] == v[a]);
  int64_t rec = 0;
  for (int64_t s = 0; s < nsteps && alive; ++s) {
    double k1v[3], k2v[3], k3v[3], k4v[3];
    // the four stages share one copy of the field evaluation (a rolled loop:
    // four inlined copies made instruction fetch the kernel's first stall)
#pragma unroll 1
    for (int stg = 0; stg < 4 && alive; ++stg) {
      double xs[3], k[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        if (stg == 0)
          xs[a] = x[a];
        else if (stg == 1)
          xs[a] = x[a] + h2 * v[a];
        else if (stg == 2)
          xs[a] = x[a] + h2 * (v[a] + h2 * k1v[a]);
        else
          xs[a] = x[a] + dt * (v[a] + h2 * k2v[a]);
      }
      alive = rk4_accel<F, MIXED>(g, kp, xs, coef, grav, k);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        if (stg == 0)
          k1v[a] = k[a];
        else if (stg == 1)
          k2v[a] = k[a];
        else if (stg == 2)
          k3v[a] = k[a];
        else
          k4v[a] = k[a];
      }
    }
    if (!alive) break;
    // position stages are v + dt/2 k1v, v + dt/2 k2v, v + dt k3v
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const double dx = v[a] + (v[a] + h2 * k1v[a]) * 2.0 + (v[a] + h2 * k2v[a]) * 2.0 + (v[a] + dt * k3v[a]);
      x[a] += h6 * dx;
      v[a] += h6 * (k1v[a] + 2.0 * k2v[a] + 2.0 * k3v[a] + k4v[a]);
    }
    if (path && rec_every > 0 && (s + 1) % rec_every == 0) {
      double *r = path + (rec * n + i) * 6;
      for (int a = 0; a < 3; ++a) {
        r[a] = x[a];
        r[3 + a] = v[a];
      }
      ++rec;
    }
  }
  if (!alive) {
    const double nan = qnan();
    for (int a = 0; a < 3; ++a) x[a] = v[a] = nan;
    atomicAdd(lost, 1ULL);
    // the remaining recorded states of a lost particle are NaN as well
    if (path && rec_every > 0)
      for (int64_t r = rec; r < nsteps / rec_every; ++r)
        for (int a = 0; a < 6; ++a) path[(r * n + i) * 6 + a] = nan;
  }
  for (int a = 0; a < 3; ++a) {
    st[a] = x[a];
    st[3 + a] = v[a];
  }
}

}  // namespace arb

using namespace arb;

extern "C" int arb_rk4_trajectories(const arb_grid *g, int32_t precision, double *state, int64_t n, double dt,
                                    int64_t nsteps, double coef, const double *gravity, double *path,
                                    int64_t record_every, unsigned long long *lost, arb_stream_t stream) {
  if (!g || !state || !lost || n < 0 || nsteps < 0 || g->dim != 3) return ARB_ERR_INVALID;
  if (g->nfield == 3) return ARB_ERR_UNSUPPORTED;  // vector mode carries no gradient
  if (path && record_every <= 0) return ARB_ERR_INVALID;
  const bool mixed = precision == ARB_PREC_MIXED;
  if (mixed ? !g->grid32 : !g->grid64) return ARB_ERR_INVALID;
  if (n == 0 || nsteps == 0) return ARB_OK;
  const double gr[3] = {gravity ? gravity[0] : 0.0, gravity ? gravity[1] : 0.0, gravity ? gravity[2] : 0.0};
  const KParams kp = make_kparams(g);
  cudaStream_t s = (cudaStream_t)stream;
  const int T = 128;
  const unsigned B = (unsigned)((n + T - 1) / T);
#define RK(FF, MX)                                                                                        \
  rk4_kernel<FF, MX><<<B, T, 0, s>>>(*g, kp, state, n, dt, nsteps, coef, gr[0], gr[1], gr[2], path, \
                                     record_every, lost)
  if (g->nfield == 1) {
    if (mixed) RK(1, true); else RK(1, false);
  } else {
    if (mixed) RK(4, true); else RK(4, false);
  }
#undef RK
  return launch_status();
}
