// A problem plugin written the way a user adds one: this file is not part
// of the library and is compiled only by the tests, which link it into a
// separate build (build(extra_plugins=[...])).  It changes no library file.
//
// The problem: one implicit Euler step of two uncoupled heat equations,
// u - dt Lap(u) = u_old and v - kappa dt Lap(v) = v_old, relaxed pointwise
// (each cell solved exactly for its own value).  Its mixed-precision
// correction form is the same linear operator on the correction.
#include "plugin_def.cuh"

namespace bsamg {

struct Heat {
  static constexpr int kKind = 40;
  static constexpr const char* kName = "heat";
  static constexpr int kNV = 2;
  static constexpr int kNParams = 2;  // dt, kappa
  static constexpr bool kCoeffsOnly = true;
  static constexpr bool kBox = false;
  static constexpr bool kMixed = true;
  static constexpr int kMxBase = 1;
  static constexpr int kMxUpdate = 1;

  static void set_params(ProbParams& pp, const double* prm, int) {
    pp.dt = prm[0];
    pp.user[0] = prm[1];
  }
  static void coefficients(const ProbParams& pp, int ndims, double h, double* c) {
    double k = 2.0 * ndims;
    c[0] = pp.dt / (h * h);
    c[1] = pp.user[0] * pp.dt / (h * h);
    c[2] = 1.0 + k * c[0];
    c[3] = 1.0 + k * c[1];
  }
  static int bc_mask(int) { return 0; }  // reflecting faces
  static int stats(int) { return 1; }

  template <int DIM>
  __device__ __forceinline__ static double nsum(const double* a, long long c, long long sy, long long sz) {
    double s = a[c - 1] + a[c + 1] + a[c - sy] + a[c + sy];
    if (DIM == 3) s = s + a[c - sz] + a[c + sz];
    return s;
  }
  template <int DIM>
  __device__ __forceinline__ static void relax(const Cell64& x, const double* cf, const ProbParams&) {
    double* u = x.q;
    double* v = u + x.sq;
    u[x.c] = (x.f[x.fc] + cf[0] * nsum<DIM>(u, x.c, x.sy, x.sz)) / cf[2];
    v[x.c] = (x.f[x.sf + x.fc] + cf[1] * nsum<DIM>(v, x.c, x.sy, x.sz)) / cf[3];
  }
  template <int DIM>
  __device__ __forceinline__ static void op(const double* a, long long c, long long sy, long long sz, long long ps,
                                            const QoldView&, const double* cf, const ProbParams&, double* r) {
    r[0] = a[c] - cf[0] * ulap<DIM>(a, c, sy, sz);
    r[1] = a[ps + c] - cf[1] * ulap<DIM>(a + ps, c, sy, sz);
  }
  // f = (u_old, v_old): both variables of qold
  template <int DIM>
  __device__ __forceinline__ static void source(const double*, long long, long long, long long, long long,
                                                const QoldView& qo, const double*, const ProbParams&, double* s) {
    s[0] = qo.p[0];
    s[1] = qo.p[qo.sq];
  }
  template <int DIM>
  __device__ __forceinline__ static void source_update(const double*, long long, long long, long long, long long,
                                                       const QoldView&, const double*, const ProbParams&,
                                                       double* su) {
    su[0] = 0.0;
    su[1] = 0.0;
  }

  static MxParams mx_params(const ProbParams&) { return MxParams{{0.f, 0.f, 0.f, 0.f}}; }
  template <int DIM>
  __device__ __forceinline__ static void mx_prep(const Cell64& x, const double* rf, float* base, float* g, int mode,
                                                 const double* cf, const ProbParams& pp) {
    base[x.fc] = (float)x.q[x.c];
    if (mode == 0) return;
    double r[2];
    if (mode == 1) {
      r[0] = rf[x.fc];
      r[1] = rf[x.sf + x.fc];
    } else {
      double o[2];
      op<DIM>(x.q, x.c, x.sy, x.sz, x.sq, QoldView{x.qold + x.c, x.sy, x.sz, x.sq}, cf, pp, o);
      r[0] = x.f[x.fc] - o[0];
      r[1] = x.f[x.sf + x.fc] - o[1];
    }
    g[x.fc] = (float)r[0];
    g[x.sf + x.fc] = (float)r[1];
  }
  template <int DIM>
  __device__ __forceinline__ static float nsum32(const float* a, long long c, long long sy, long long sz) {
    float s = a[c - 1] + a[c + 1] + a[c - sy] + a[c + sy];
    if (DIM == 3) s = s + a[c - sz] + a[c + sz];
    return s;
  }
  template <int DIM, typename T>
  __device__ __forceinline__ static void mx_relax(const Cell32& x, const T* cf, const MxParams&) {
    float* u = x.e;
    float* v = u + x.sq;
    u[x.c] = (float)((T(x.g[x.fc]) + cf[0] * T(nsum32<DIM>(u, x.c, x.sy, x.sz))) / cf[2]);
    v[x.c] = (float)((T(x.g[x.sf + x.fc]) + cf[1] * T(nsum32<DIM>(v, x.c, x.sy, x.sz))) / cf[3]);
  }
  template <int DIM>
  __device__ __forceinline__ static void mx_op(const float* e, long long c, long long sy, long long sz, long long ps,
                                               const float*, long long, long long, const float* cf, const MxParams&,
                                               float* m) {
    m[0] = e[c] - cf[0] * ulap<DIM>(e, c, sy, sz);
    m[1] = e[ps + c] - cf[1] * ulap<DIM>(e + ps, c, sy, sz);
  }
};

BSAMG_PLUGIN(Heat)

}  // namespace bsamg
