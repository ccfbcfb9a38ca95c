// FP64 face/cell kernels of the steady SIMPLE iteration: geometry, boundary conditions,
// Green-Gauss gradients, momentum / pressure-correction / scalar assembly, Rhie-Chow
// fluxes and corrections.
//
// Design: owner-computes.  Every kernel that produces a per-cell quantity runs one thread
// per cell and gathers over that cell's faces in the reference's own order (Cell[i].face[]
// for assembly, ascending face index for gradients), so no atomics are needed, results are
// reproducible, and -- because this translation unit is compiled with -fmad=false -- every
// product and sum is rounded exactly where the reference's source rounds it: the outputs
// are bit-identical to the reference arithmetic evaluated without contraction.
#include <cuda_runtime.h>

#include <type_traits>

#include "cycas_device.h"

namespace cycas {

namespace {

constexpr int kThreads = 256;
constexpr double SMALL = 1.e-16;  // NS/BasicType.h:12

inline int blocks_for(long n) { return (int)((n + kThreads - 1) / kThreads); }

__device__ __forceinline__ double dmin(double x, double y) { return x < y ? x : y; }  // CYCASMIN

// vec_dot / vec_len with the reference's summation order (tools.cpp:22-36)
__device__ __forceinline__ double vdot3(const double* a, double b0, double b1, double b2) {
  double s = 0.;
  s += a[0] * b0;
  s += a[1] * b1;
  s += a[2] * b2;
  return s;
}
__device__ __forceinline__ double vdot3v(double a0, double a1, double a2, double b0, double b1, double b2) {
  double s = 0.;
  s += a0 * b0;
  s += a1 * b1;
  s += a2 * b2;
  return s;
}
// the same sums in the arithmetic type T of an assembly kernel (double: the functions above)
template <class T>
__device__ __forceinline__ T tmin(T x, T y) { return x < y ? x : y; }
template <class T>
__device__ __forceinline__ T tdot3(const T* a, T b0, T b1, T b2) {
  T s = T(0);
  s += a[0] * b0;
  s += a[1] * b1;
  s += a[2] * b2;
  return s;
}
template <class T>
__device__ __forceinline__ T tdot3v(T a0, T a1, T a2, T b0, T b1, T b2) {
  T s = T(0);
  s += a0 * b0;
  s += a1 * b1;
  s += a2 * b2;
  return s;
}

// ------------------------------------------------------------------ geometry
// Tri3DArea / TetVolum (geometry.cpp:365-383)
__device__ double tri_area(const double* x1, const double* x2, const double* x3) {
  double v1[3], v2[3];
  for (int i = 0; i < 3; i++) {
    v1[i] = x2[i] - x1[i];
    v2[i] = x3[i] - x1[i];
  }
  double a1 = v1[1] * v2[2] - v1[2] * v2[1];
  double a2 = -v1[0] * v2[2] + v1[2] * v2[0];
  double a3 = v1[0] * v2[1] - v1[1] * v2[0];
  return 0.5 * sqrt(a1 * a1 + a2 * a2 + a3 * a3);
}
__device__ double tet_vol(const double* x1, const double* x2, const double* x3, const double* x4) {
  double d1[3], d2[3], d3[3], v[3];
  for (int i = 0; i < 3; i++) {
    d1[i] = x2[i] - x1[i];
    d2[i] = x3[i] - x1[i];
    d3[i] = x4[i] - x1[i];
  }
  v[0] = d1[1] * d2[2] - d1[2] * d2[1];
  v[1] = -d1[0] * d2[2] + d1[2] * d2[0];
  v[2] = d1[0] * d2[1] - d1[1] * d2[0];
  return 1. / 6. * fabs(vdot3(v, d3[0], d3[1], d3[2]));
}

// cell volume and centre: six tetrahedra of the hex-form cell (geometry.cpp:416-459)
__global__ void k_cell_geometry(int ncel, const int* __restrict__ cv, const double* __restrict__ X,
                                double* __restrict__ vol, double* __restrict__ cx) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncel) return;
  double x[8][3];
  for (int k = 0; k < 8; k++) {
    int v = cv[8 * (long)i + k];
    for (int d = 0; d < 3; d++) x[k][d] = X[3 * (long)v + d];
  }
  double V1 = tet_vol(x[0], x[1], x[3], x[5]);
  double V2 = tet_vol(x[0], x[4], x[3], x[5]);
  double V3 = tet_vol(x[3], x[4], x[7], x[5]);
  double V4 = tet_vol(x[1], x[2], x[3], x[6]);
  double V5 = tet_vol(x[1], x[5], x[3], x[6]);
  double V6 = tet_vol(x[7], x[3], x[5], x[6]);
  vol[i] = V1 + V2 + V3 + V4 + V5 + V6;
  double Vsum = V1 + V2 + V3 + V4 + V5 + V6;
  for (int j = 0; j < 3; j++) {
    double xc1 = 0.25 * (x[0][j] + x[1][j] + x[3][j] + x[5][j]);
    double xc2 = 0.25 * (x[0][j] + x[4][j] + x[3][j] + x[5][j]);
    double xc3 = 0.25 * (x[3][j] + x[4][j] + x[7][j] + x[5][j]);
    double xc4 = 0.25 * (x[1][j] + x[2][j] + x[3][j] + x[6][j]);
    double xc5 = 0.25 * (x[1][j] + x[5][j] + x[3][j] + x[6][j]);
    double xc6 = 0.25 * (x[7][j] + x[3][j] + x[5][j] + x[6][j]);
    cx[3 * (long)i + j] = 1. / Vsum * (V1 * xc1 + V2 * xc2 + V3 * xc3 + V4 * xc4 + V5 * xc5 + V6 * xc6);
  }
}

// face centre, area vector oriented cell1 -> cell2, area, lambda (geometry.cpp:561-624)
__global__ void k_face_geometry(int nfac, const int* __restrict__ fv, const double* __restrict__ X,
                                const int* __restrict__ c1, const int* __restrict__ c2,
                                const double* __restrict__ cx, double* __restrict__ fx, double* __restrict__ fn,
                                double* __restrict__ farea, double* __restrict__ flam, int* err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nfac) return;
  const double *v1 = X + 3 * (long)fv[4 * (long)i], *v2 = X + 3 * (long)fv[4 * (long)i + 1],
               *v3 = X + 3 * (long)fv[4 * (long)i + 2], *v4 = X + 3 * (long)fv[4 * (long)i + 3];
  double area1 = tri_area(v1, v2, v4);
  double area2 = tri_area(v2, v3, v4);
  double x[3], n[3];
  for (int j = 0; j < 3; j++) {
    double xc1 = 1. / 3 * (v1[j] + v2[j] + v4[j]);
    double xc2 = 1. / 3 * (v2[j] + v3[j] + v4[j]);
    x[j] = (area1 * xc1 + area2 * xc2) / (area1 + area2);
  }
  double d1[3], d2[3];
  for (int j = 0; j < 3; j++) {
    d1[j] = v1[j] - v3[j];
    d2[j] = v2[j] - v4[j];
  }
  n[0] = d1[1] * d2[2] - d1[2] * d2[1];
  n[1] = -d1[0] * d2[2] + d1[2] * d2[0];
  n[2] = d1[0] * d2[1] - d1[1] * d2[0];
  for (int j = 0; j < 3; j++) n[j] = 0.5 * n[j];
  int a = c1[i];
  const double* xa = cx + 3 * (long)a;
  if (vdot3(n, x[0] - xa[0], x[1] - xa[1], x[2] - xa[2]) < 0.)
    for (int j = 0; j < 3; j++) n[j] = -n[j];
  double ar = sqrt(vdot3(n, n[0], n[1], n[2]));
  if (fabs((area1 + area2 - ar) / ar) > 1.e-4) atomicOr(err, 2);
  int b = c2[i];
  double lam = 1.;
  if (b >= 0) {
    const double* xb = cx + 3 * (long)b;
    double e1[3] = {x[0] - xa[0], x[1] - xa[1], x[2] - xa[2]};
    double e2[3] = {x[0] - xb[0], x[1] - xb[1], x[2] - xb[2]};
    double r1 = sqrt(vdot3(e1, e1[0], e1[1], e1[2]));
    double r2 = sqrt(vdot3(e2, e2[0], e2[1], e2[2]));
    lam = r2 / (r1 + r2);
  }
  for (int j = 0; j < 3; j++) {
    fx[3 * (long)i + j] = x[j];
    fn[3 * (long)i + j] = n[j];
  }
  farea[i] = ar;
  flam[i] = lam;
}

// rlencos, auxiliary points (geometry.cpp:671-705) and wall distance (geometry.cpp:657-669)
__global__ void k_face_geometry2(int nfac, const int* __restrict__ c1, const int* __restrict__ c2,
                                 const int* __restrict__ fbnd, const double* __restrict__ cx,
                                 const double* __restrict__ fx, const double* __restrict__ fn,
                                 const double* __restrict__ farea, double* __restrict__ rlencos,
                                 double* __restrict__ xpac, double* __restrict__ xnac,
                                 double* __restrict__ bdist, int* err) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nfac) return;
  const double* x = fx + 3 * (long)i;
  const double* n = fn + 3 * (long)i;
  double ar = farea[i];
  int a = c1[i], b = c2[i];
  const double* xa = cx + 3 * (long)a;
  if (b == -10) {
    double dx[3] = {x[0] - xa[0], x[1] - xa[1], x[2] - xa[2]};
    rlencos[i] = ar / (vdot3(dx, n[0], n[1], n[2]) / ar);
    double dist = vdot3(dx, n[0], n[1], n[2]) / ar;
    bdist[fbnd[i]] = dist;
    if (dist < 0.) atomicOr(err, 2);
    for (int j = 0; j < 3; j++) xpac[3 * (long)i + j] = xnac[3 * (long)i + j] = 0.0;
  } else {
    const double* xb = cx + 3 * (long)b;
    double dx[3] = {xb[0] - xa[0], xb[1] - xa[1], xb[2] - xa[2]};
    rlencos[i] = ar / fabs(vdot3(dx, n[0], n[1], n[2]) / ar);
    double d[3] = {x[0] - xa[0], x[1] - xa[1], x[2] - xa[2]};
    double ss = vdot3(d, n[0], n[1], n[2]) / ar;
    for (int j = 0; j < 3; j++) d[j] = ss * n[j] / ar;
    for (int j = 0; j < 3; j++) xpac[3 * (long)i + j] = x[j] - d[j];
    double e[3] = {x[0] - xb[0], x[1] - xb[1], x[2] - xb[2]};
    ss = vdot3(e, n[0], n[1], n[2]) / ar;
    for (int j = 0; j < 3; j++) e[j] = ss * n[j] / ar;
    for (int j = 0; j < 3; j++) xnac[3 * (long)i + j] = x[j] - e[j];
  }
}

// ------------------------------------------------------------------ boundary conditions
// SetBCVelocity per-face part (navier_bc.cpp:13-60) and, optionally, SetBCPressure
// (navier_bc.cpp:121-155): every non-periodic boundary copies the owner-cell pressure.
__global__ void k_bc_velocity(int nbnd, const int* __restrict__ b_face, const int* __restrict__ b_type,
                              const int* __restrict__ f_c1, const double* __restrict__ f_n,
                              const double* __restrict__ f_area, const double* __restrict__ R,
                              const double* __restrict__ U, const double* __restrict__ V,
                              const double* __restrict__ W, const double* __restrict__ P, double* BRo, double* BU,
                              double* BV, double* BW, double* BPre, int set_pressure) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbnd) return;
  int iface = b_face[i];
  int ic = f_c1[iface];
  switch (b_type[i]) {
    case 1:
      BRo[i] = R[ic];
      BU[i] = 0.;
      BV[i] = 0.;
      BW[i] = 0.;
      break;
    case 3:
      BRo[i] = R[ic];
      BU[i] = U[ic];
      BV[i] = V[ic];
      BW[i] = W[ic];
      break;
    case 4: {
      double ar = f_area[iface];
      double s1 = f_n[3 * (long)iface] / ar, s2 = f_n[3 * (long)iface + 1] / ar, s3 = f_n[3 * (long)iface + 2] / ar;
      double un = U[ic] * s1 + V[ic] * s2 + W[ic] * s3;
      BU[i] = U[ic] - un * s1;
      BV[i] = V[ic] - un * s2;
      BW[i] = W[ic] - un * s3;
      BRo[i] = R[ic];
      break;
    }
    default:  // inlet keeps its prescribed values
      break;
  }
  if (set_pressure) BPre[i] = P[ic];
}

// Outlet mass-flow correction (navier_bc.cpp:62-118).  The three sums are accumulated in
// boundary order by one thread, exactly as the reference's serial loop; the other threads
// compute the per-face terms in chunks and then rescale the outlet faces.
__global__ void k_bc_outlet(int n_in, const int* __restrict__ in_list, int n_out, const int* __restrict__ out_list,
                            const int* __restrict__ b_face, const double* __restrict__ f_n,
                            const double* __restrict__ f_area, double* BRo, double* BU, double* BV, double* BW,
                            const int* __restrict__ in0, const int* __restrict__ out0) {
  // batches: block c takes the inlet and outlet boundaries of case c (in0/out0 ranges)
  if (in0) {
    in_list += in0[blockIdx.x];
    n_in = in0[blockIdx.x + 1] - in0[blockIdx.x];
    out_list += out0[blockIdx.x];
    n_out = out0[blockIdx.x + 1] - out0[blockIdx.x];
    if (n_out == 0) return;
  }
  // terms of both lists in shared memory, then the three serial sums on three warps at once
  // (each sum is one dependent chain of FP64 additions; running them side by side hides two)
  __shared__ double iterm[kThreads], oterm[kThreads], aterm[kThreads];
  __shared__ double s_min, s_mout, s_aout;
  if (threadIdx.x == 0) s_min = s_mout = s_aout = 0.0;
  const int cmax = max(n_in, n_out);
  for (int base = 0; base < cmax; base += kThreads) {
    __syncthreads();
    const int k = base + threadIdx.x;
    if (k < n_in) {
      const int i = in_list[k];
      const double* n = f_n + 3 * (long)b_face[i];
      iterm[threadIdx.x] = BRo[i] * (BU[i] * n[0] + BV[i] * n[1] + BW[i] * n[2]);
    }
    if (k < n_out) {
      const int i = out_list[k];
      const double* n = f_n + 3 * (long)b_face[i];
      oterm[threadIdx.x] = BRo[i] * (BU[i] * n[0] + BV[i] * n[1] + BW[i] * n[2]);
      aterm[threadIdx.x] = BRo[i] * f_area[i];  // Face[i] with the boundary index, as written
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0 && threadIdx.x < 96) {
      const int w = threadIdx.x >> 5;
      const int cnt = w == 0 ? n_in : n_out;
      const int lim = min(kThreads, cnt - base);
      const double* t = w == 0 ? iterm : (w == 1 ? oterm : aterm);
      double acc = w == 0 ? s_min : (w == 1 ? s_mout : s_aout);
      for (int q = 0; q < lim; q++) acc += t[q];
      if (w == 0) s_min = acc;
      else if (w == 1) s_mout = acc;
      else s_aout = acc;
    }
  }
  __syncthreads();
  double mflowin = s_min, mflowout = s_mout, aout = s_aout;
  if (fabs(mflowout) > SMALL) {
    double rate = -mflowin / mflowout;
    for (int k = threadIdx.x; k < n_out; k += blockDim.x) {
      int iface = b_face[out_list[k]];  // BU[iface]: boundary faces come first, iface == bnd index
      BU[iface] *= rate;
      BV[iface] *= rate;
      BW[iface] *= rate;
    }
  } else {
    double rate = (-mflowin - mflowout) / aout;
    for (int k = threadIdx.x; k < n_out; k += blockDim.x) {
      int iface = b_face[out_list[k]];
      const double* n = f_n + 3 * (long)iface;
      double ar = f_area[iface];
      BU[iface] += rate * n[0] / ar;
      BV[iface] += rate * n[1] / ar;
      BW[iface] += rate * n[2] / ar;
    }
  }
}

// SetBCDeltaP (navier_bc.cpp:157-181)
__global__ void k_bc_copy(int nbnd, const int* __restrict__ b_face, const int* __restrict__ f_c1,
                          const double* __restrict__ cellv, double* __restrict__ bv) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbnd) return;
  bv[i] = cellv[f_c1[b_face[i]]];
}

// ------------------------------------------------------------------ gradient
template <int NF>
struct GradArgs {
  const double* phi[NF];
  const double* bphi[NF];
  double* grad[NF];
};

// Green-Gauss (navier_gradient.cpp:12-74, limiter 0): the reference loops over faces and
// scatters +-pf*n to both cells; per cell that is a sum over its faces in ascending face
// index, which is the order c_gface holds.
// T is the arithmetic type: double in the FP64 path (bit-exact with the reference), float in
// mixed-precision contexts (loads are rounded to float once, results widened back).
template <class T, int NF>
__global__ void k_gradient(int ncel, const int* __restrict__ c_nface, const int* __restrict__ c_gface,
                           const int* __restrict__ f_c1, const int* __restrict__ f_c2,
                           const int* __restrict__ f_bnd, const double* __restrict__ f_lambda,
                           const double* __restrict__ f_n, const double* __restrict__ c_vol, GradArgs<NF> a) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncel) return;
  T g[NF][3];
#pragma unroll
  for (int q = 0; q < NF; q++) g[q][0] = g[q][1] = g[q][2] = T(0);
  int nf = c_nface[i];
  for (int k = 0; k < nf; k++) {
    int fid = c_gface[(long)k * ncel + i];
    int c1 = f_c1[fid], c2 = f_c2[fid];
    T n0 = (T)f_n[3 * (long)fid], n1 = (T)f_n[3 * (long)fid + 1], n2 = (T)f_n[3 * (long)fid + 2];
    if (c2 >= 0) {
      T lam = (T)f_lambda[fid];
      bool own = (c1 == i);
#pragma unroll
      for (int q = 0; q < NF; q++) {
        T pf;
        if constexpr (std::is_same<T, float>::value) {
          // FP32: the face value relative to the cell's own, lambda-weighted difference of the
          // FP64 values (the cell's normals sum to zero, so the sum is the same while the large
          // face values no longer cancel in FP32)
          const double d = __ldg(a.phi[q] + (own ? c2 : c1)) - __ldg(a.phi[q] + i);
          pf = own ? (T(1) - lam) * (T)d : lam * (T)d;
        } else {
          pf = lam * (T)__ldg(a.phi[q] + c1) + (T(1) - lam) * (T)__ldg(a.phi[q] + c2);
        }
        if (own) {
          g[q][0] += pf * n0;
          g[q][1] += pf * n1;
          g[q][2] += pf * n2;
        } else {
          g[q][0] -= pf * n0;
          g[q][1] -= pf * n1;
          g[q][2] -= pf * n2;
        }
      }
    } else {
      int b = f_bnd[fid];
#pragma unroll
      for (int q = 0; q < NF; q++) {
        T pf;
        if constexpr (std::is_same<T, float>::value) pf = (T)(__ldg(a.bphi[q] + b) - __ldg(a.phi[q] + i));
        else pf = (T)__ldg(a.bphi[q] + b);
        g[q][0] += pf * n0;
        g[q][1] += pf * n1;
        g[q][2] += pf * n2;
      }
    }
  }
  T vol = (T)c_vol[i];
#pragma unroll
  for (int q = 0; q < NF; q++)
    for (int d = 0; d < 3; d++) a.grad[q][3 * (long)i + d] = (double)(g[q][d] / vol);
}

// ------------------------------------------------------------------ momentum
struct MomArgs {
  int ncel;
  const int *c_nface, *c_face, *c_slot, *c_diag;
  const int *f_c1, *f_c2, *f_bnd, *b_type;
  const double *f_x, *f_n, *f_lambda, *f_rlencos, *c_x, *c_vol;
  const double *U, *V, *W, *P, *R, *VisLam, *VisTur, *RUFace;
  const double *dU, *dV, *dW, *dP, *BU, *BV, *BW;
  double *A, *bu, *bv, *bw, *Apr, *dinv, *old, *shear;
  double urf0, g0, g1, g2;
  int* warn;
  const double *Unp, *Vnp, *Wnp;  // previous time level (scheme != 0)
  int scheme;                     // 0 steady, 1 Euler, 2 second-order form
  double dt;
};

// BuildVelocityMatrix cell loop (navier_velocity.cpp:100-383)
// T as for k_gradient: double (bit-exact) or float (mixed-precision contexts).
template <class T>
__global__ void __launch_bounds__(kThreads) k_momentum(MomArgs a) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.ncel) return;
  const long N = a.ncel;
  T Ui = (T)a.U[i], Vi = (T)a.V[i], Wi = (T)a.W[i];
  T xi0 = (T)a.c_x[3 * i], xi1 = (T)a.c_x[3 * i + 1], xi2 = (T)a.c_x[3 * i + 2];
  T visi = (T)a.VisLam[i] + (T)a.VisTur[i];
  T gu[3] = {(T)a.dU[3 * i], (T)a.dU[3 * i + 1], (T)a.dU[3 * i + 2]};
  T gv[3] = {(T)a.dV[3 * i], (T)a.dV[3 * i + 1], (T)a.dV[3 * i + 2]};
  T gw[3] = {(T)a.dW[3 * i], (T)a.dW[3 * i + 1], (T)a.dW[3 * i + 2]};
  T app = T(0), su = T(0), sv = T(0), sw = T(0);
  if (a.scheme != 0) {  // unsteady terms (navier_velocity.cpp:108-123)
    T coef = (T)a.R[i] / (T)a.dt * (T)a.c_vol[i];
    T un = (T)a.Unp[i], vn = (T)a.Vnp[i], wn = (T)a.Wnp[i];
    if (a.scheme == 1) {
      app += coef;
      su += coef * un;
      sv += coef * vn;
      sw += coef * wn;
    } else {  // both previous levels hold the same values (SaveTransientOldData)
      app += T(1.5) * coef;
      su += coef * (T(2) * un - T(0.5) * un);
      sv += coef * (T(2) * vn - T(0.5) * vn);
      sw += coef * (T(2) * wn - T(0.5) * wn);
    }
  }
  int nf = a.c_nface[i];
  for (int j = 0; j < nf; j++) {
    int iface = a.c_face[j * N + i];
    int ip = a.f_c1[iface], in = a.f_c2[iface];
    T fde0, fde1, fde2, fdi0, fdi1, fdi2, fcs0, fcs1, fcs2;
    const double* fn = a.f_n + 3 * (long)iface;
    const double* fx = a.f_x + 3 * (long)iface;
    if (in < 0) {
      int bnd = a.f_bnd[iface];
      int t = a.b_type[bnd];
      T s1 = (T)fn[0], s2 = (T)fn[1], s3 = (T)fn[2];
      T RUn = (T)a.RUFace[iface];
      T Visc = visi;
      T dudx = gu[0], dudy = gu[1], dudz = gu[2];
      T dvdx = gv[0], dvdy = gv[1], dvdz = gv[2];
      T dwdx = gw[0], dwdy = gw[1], dwdz = gw[2];
      T dxc0 = (T)fx[0] - xi0, dxc1 = (T)fx[1] - xi1, dxc2 = (T)fx[2] - xi2;
      T val = Visc * (T)a.f_rlencos[iface];
      app += val;
      if (t == 1) {
        T sh0 = (dudx + dudx) * s1 + (dudy + dvdx) * s2 + (dudz + dwdx) * s3;
        T sh1 = (dvdx + dudy) * s1 + (dvdy + dvdy) * s2 + (dvdz + dwdy) * s3;
        T sh2 = (dwdx + dudz) * s1 + (dwdy + dvdz) * s2 + (dwdz + dwdz) * s3;
        sh0 *= Visc;
        sh1 *= Visc;
        sh2 *= Visc;
        T Pi = (T)a.P[i];
        sh0 += Pi * s1;
        sh1 += Pi * s2;
        sh2 += Pi * s3;
        a.shear[3 * (long)bnd] = sh0;
        a.shear[3 * (long)bnd + 1] = sh1;
        a.shear[3 * (long)bnd + 2] = sh2;
        fde0 = val * Ui;
        fde1 = val * Vi;
        fde2 = val * Wi;
        fdi0 = val * Ui;
        fdi1 = val * Vi;
        fdi2 = val * Wi;
        fcs0 = fcs1 = fcs2 = T(0);
      } else {
        fde0 = (dudx + dudx) * s1 + (dudy + dvdx) * s2 + (dudz + dwdx) * s3;
        fde1 = (dvdx + dudy) * s1 + (dvdy + dvdy) * s2 + (dvdz + dwdy) * s3;
        fde2 = (dwdx + dudz) * s1 + (dwdy + dvdz) * s2 + (dwdz + dwdz) * s3;
        fde0 *= Visc;
        fde1 *= Visc;
        fde2 *= Visc;
        T bu = (T)a.BU[bnd], bv = (T)a.BV[bnd], bw = (T)a.BW[bnd];
        fdi0 = val * (dudx * dxc0 + dudy * dxc1 + dudz * dxc2 - bu);
        fdi1 = val * (dvdx * dxc0 + dvdy * dxc1 + dvdz * dxc2 - bv);
        fdi2 = val * (dwdx * dxc0 + dwdy * dxc1 + dwdz * dxc2 - bw);
        if (t == 4) {
          fcs0 = fcs1 = fcs2 = T(0);
        } else {  // 2 inlet, 3 outlet
          if (t == 2 && RUn > T(0)) atomicAdd(a.warn, 1);
          T fl = tmin<T>(RUn, T(0));
          app -= fl;
          fcs0 = fl * bu;
          fcs1 = fl * bv;
          fcs2 = fl * bw;
        }
      }
    } else {
      T s1, s2, s3, RUn, lam;
      T fl0 = (T)a.f_lambda[iface];
      if (i != ip) {
        in = ip;
        s1 = -(T)fn[0];
        s2 = -(T)fn[1];
        s3 = -(T)fn[2];
        RUn = -(T)a.RUFace[iface];
        lam = T(1) - fl0;
      } else {
        s1 = (T)fn[0];
        s2 = (T)fn[1];
        s3 = (T)fn[2];
        RUn = (T)a.RUFace[iface];
        lam = fl0;
      }
      T lam2 = T(1) - lam;
      T visn = (T)a.VisLam[in] + (T)a.VisTur[in];
      T Visc = lam * visi + lam2 * visn;
      T nu0 = (T)a.dU[3 * (long)in], nu1 = (T)a.dU[3 * (long)in + 1], nu2 = (T)a.dU[3 * (long)in + 2];
      T nv0 = (T)a.dV[3 * (long)in], nv1 = (T)a.dV[3 * (long)in + 1], nv2 = (T)a.dV[3 * (long)in + 2];
      T nw0 = (T)a.dW[3 * (long)in], nw1 = (T)a.dW[3 * (long)in + 1], nw2 = (T)a.dW[3 * (long)in + 2];
      T dudx = lam * gu[0] + lam2 * nu0, dudy = lam * gu[1] + lam2 * nu1, dudz = lam * gu[2] + lam2 * nu2;
      T dvdx = lam * gv[0] + lam2 * nv0, dvdy = lam * gv[1] + lam2 * nv1, dvdz = lam * gv[2] + lam2 * nv2;
      T dwdx = lam * gw[0] + lam2 * nw0, dwdy = lam * gw[1] + lam2 * nw1, dwdz = lam * gw[2] + lam2 * nw2;
      T apn = T(0);
      if (RUn < T(0)) {
        apn += RUn;
        app -= RUn;
      }
      T val = Visc * (T)a.f_rlencos[iface];
      app += val;
      apn += -val;
      a.A[a.c_slot[j * N + i]] = apn;
      T Un = (T)a.U[in], Vn = (T)a.V[in], Wn = (T)a.W[in];
      T xn0 = (T)a.c_x[3 * (long)in], xn1 = (T)a.c_x[3 * (long)in + 1], xn2 = (T)a.c_x[3 * (long)in + 2];
      T ufi, vfi, wfi, ufh, vfh, wfh, cu, cv, cw;
      if (RUn > T(0)) {
        ufi = Ui;
        vfi = Vi;
        wfi = Wi;
        T dx0 = (T)fx[0] - xi0, dx1 = (T)fx[1] - xi1, dx2 = (T)fx[2] - xi2;
        cu = tdot3<T>(gu, dx0, dx1, dx2);
        cv = tdot3<T>(gv, dx0, dx1, dx2);
        cw = tdot3<T>(gw, dx0, dx1, dx2);
        ufh = Ui + cu;
        vfh = Vi + cv;
        wfh = Wi + cw;
      } else {
        ufi = Un;
        vfi = Vn;
        wfi = Wn;
        T dx0 = (T)fx[0] - xn0, dx1 = (T)fx[1] - xn1, dx2 = (T)fx[2] - xn2;
        cu = tdot3v<T>(nu0, nu1, nu2, dx0, dx1, dx2);
        cv = tdot3v<T>(nv0, nv1, nv2, dx0, dx1, dx2);
        cw = tdot3v<T>(nw0, nw1, nw2, dx0, dx1, dx2);
        ufh = Un + cu;
        vfh = Vn + cv;
        wfh = Wn + cw;
      }
      if constexpr (std::is_same<T, float>::value) {
        // FP32: the high-order correction itself (ufh - ufi is exactly the gradient term, whose
        // digits the FP32 subtraction from ufh would lose)
        fcs0 = RUn * cu;
        fcs1 = RUn * cv;
        fcs2 = RUn * cw;
      } else {
        fcs0 = RUn * (ufh - ufi);
        fcs1 = RUn * (vfh - vfi);
        fcs2 = RUn * (wfh - wfi);
      }
      fde0 = (dudx + dudx) * s1 + (dudy + dvdx) * s2 + (dudz + dwdx) * s3;
      fde1 = (dvdx + dudy) * s1 + (dvdy + dvdy) * s2 + (dvdz + dwdy) * s3;
      fde2 = (dwdx + dudz) * s1 + (dwdy + dvdz) * s2 + (dwdz + dwdz) * s3;
      fde0 *= Visc;
      fde1 *= Visc;
      fde2 *= Visc;
      T dxc0 = xn0 - xi0, dxc1 = xn1 - xi1, dxc2 = xn2 - xi2;
      fdi0 = val * (dudx * dxc0 + dudy * dxc1 + dudz * dxc2);
      fdi1 = val * (dvdx * dxc0 + dvdy * dxc1 + dvdz * dxc2);
      fdi2 = val * (dwdx * dxc0 + dwdy * dxc1 + dwdz * dxc2);
    }
    su += fde0 - fdi0 - fcs0;
    sv += fde1 - fdi1 - fcs1;
    sw += fde2 - fdi2 - fcs2;
  }
  app /= (T)a.urf0;
  T apr = T(1) / (app);
  a.Apr[i] = apr;
  a.dinv[i] = apr;
  a.A[a.c_diag[i]] = app;
  T vol = (T)a.c_vol[i];
  T Ri = (T)a.R[i];
  a.bu[i] = su + (T(1) - (T)a.urf0) * app * Ui + (-(T)a.dP[3 * i] + Ri * (T)a.g0) * vol;
  a.bv[i] = sv + (T(1) - (T)a.urf0) * app * Vi + (-(T)a.dP[3 * i + 1] + Ri * (T)a.g1) * vol;
  a.bw[i] = sw + (T(1) - (T)a.urf0) * app * Wi + (-(T)a.dP[3 * i + 2] + Ri * (T)a.g2) * vol;
  a.old[i] = a.U[i];  // the FP64 field itself (the residual compares with it exactly)
  a.old[N + i] = a.V[i];
  a.old[2 * N + i] = a.W[i];
}

// ------------------------------------------------------------------ Rhie-Chow
// CalRUFace2 (navier_velocity.cpp:425-477); T as for k_gradient
template <class T>
__global__ void k_ruface2(int nfac, const int* __restrict__ f_c1, const int* __restrict__ f_c2,
                          const int* __restrict__ f_bnd, const double* __restrict__ f_n,
                          const double* __restrict__ f_area, const double* __restrict__ f_lambda,
                          const double* __restrict__ f_xpac, const double* __restrict__ f_xnac,
                          const double* __restrict__ c_x, const double* __restrict__ c_vol,
                          const double* __restrict__ R, const double* __restrict__ U, const double* __restrict__ V,
                          const double* __restrict__ W, const double* __restrict__ P,
                          const double* __restrict__ Apr, const double* __restrict__ dP,
                          const double* __restrict__ BRo, const double* __restrict__ BU,
                          const double* __restrict__ BV, const double* __restrict__ BW, double* __restrict__ RUFace) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nfac) return;
  int c1 = f_c1[i], c2 = f_c2[i];
  const double* n = f_n + 3 * (long)i;
  const T n0 = (T)n[0], n1 = (T)n[1], n2 = (T)n[2];
  if (c2 < 0) {
    int b = f_bnd[i];
    T ro = (T)BRo[b];
    T ruf = (T)BU[b] * ro, rvf = (T)BV[b] * ro, rwf = (T)BW[b] * ro;
    RUFace[i] = (double)(ruf * n0 + rvf * n1 + rwf * n2);
    return;
  }
  T lam = (T)f_lambda[i], lam2 = T(1) - lam;
  T R1 = (T)R[c1], R2 = (T)R[c2];
  T rf = lam * R1 + lam2 * R2;
  T ruf = lam * R1 * (T)U[c1] + lam2 * R2 * (T)U[c2];
  T rvf = lam * R1 * (T)V[c1] + lam2 * R2 * (T)V[c2];
  T rwf = lam * R1 * (T)W[c1] + lam2 * R2 * (T)W[c2];
  T ru = ruf * n0 + rvf * n1 + rwf * n2;
  const double* xp = f_xpac + 3 * (long)i;
  const double* xn = f_xnac + 3 * (long)i;
  const double* x1 = c_x + 3 * (long)c1;
  const double* x2 = c_x + 3 * (long)c2;
  const T g1[3] = {(T)dP[3 * (long)c1], (T)dP[3 * (long)c1 + 1], (T)dP[3 * (long)c1 + 2]};
  const T g2[3] = {(T)dP[3 * (long)c2], (T)dP[3 * (long)c2 + 1], (T)dP[3 * (long)c2 + 2]};
  const T xp0 = (T)xp[0], xp1 = (T)xp[1], xp2 = (T)xp[2], xn0 = (T)xn[0], xn1 = (T)xn[1], xn2 = (T)xn[2];
  T P1, P2;
  if constexpr (std::is_same<T, float>::value) {
    // FP32: the two face pressures relative to P[c1], the cell difference taken in FP64 (only
    // P2 - P1 enters the flux, and P itself carries an offset that would swamp it in FP32)
    P1 = tdot3<T>(g1, xp0 - (T)x1[0], xp1 - (T)x1[1], xp2 - (T)x1[2]);
    P2 = (T)(P[c2] - P[c1]) + tdot3<T>(g2, xn0 - (T)x2[0], xn1 - (T)x2[1], xn2 - (T)x2[2]);
  } else {
    P1 = (T)P[c1] + tdot3<T>(g1, xp0 - (T)x1[0], xp1 - (T)x1[1], xp2 - (T)x1[2]);
    P2 = (T)P[c2] + tdot3<T>(g2, xn0 - (T)x2[0], xn1 - (T)x2[1], xn2 - (T)x2[2]);
  }
  T dx0 = xn0 - xp0, dx1 = xn1 - xp1, dx2 = xn2 - xp2;
  T d12 = sqrt(tdot3v<T>(dx0, dx1, dx2, dx0, dx1, dx2));
  T aprf = lam * (T)Apr[c1] + lam2 * (T)Apr[c2];
  T vol = lam * (T)c_vol[c1] + lam2 * (T)c_vol[c2];
  T dpx = lam * g1[0] + lam2 * g2[0];
  T dpy = lam * g1[1] + lam2 * g2[1];
  T dpz = lam * g1[2] + lam2 * g2[2];
  T dpn = dpx * dx0 + dpy * dx1 + dpz * dx2;
  ru -= rf * (T)f_area[i] * aprf / d12 * vol * ((P2 - P1) - dpn);
  RUFace[i] = (double)ru;
}

// ------------------------------------------------------------------ pressure correction
// BuildPressureMatrix, constant density (navier_pressure.cpp:106-224)
__global__ void k_pressure(int ncel, const int* __restrict__ c_nface, const int* __restrict__ c_face,
                           const int* __restrict__ c_slot, const int* __restrict__ c_diag,
                           const int* __restrict__ f_c1, const int* __restrict__ f_c2,
                           const double* __restrict__ f_lambda, const double* __restrict__ f_rlencos,
                           const double* __restrict__ c_vol, const double* __restrict__ R,
                           const double* __restrict__ Apr, const double* __restrict__ RUFace, double* __restrict__ A,
                           double* __restrict__ bp, double* __restrict__ dinv) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncel) return;
  const long N = ncel;
  double valcen = 0., bpv = 0.;
  double rai = R[i] * Apr[i];
  double voli = c_vol[i];
  int nf = c_nface[i];
  for (int j = 0; j < nf; j++) {
    int iface = c_face[j * N + i];
    int c1 = f_c1[iface], c2 = f_c2[iface];
    bool own = (i == c1);
    if (own) bpv += RUFace[iface];
    else bpv -= RUFace[iface];
    int in = own ? c2 : c1;
    if (c2 < 0) continue;
    double lam = own ? f_lambda[iface] : 1. - f_lambda[iface];
    double lam2 = 1. - lam;
    double roapf = rai * lam + R[in] * Apr[in] * lam2;
    double vol = voli * lam + c_vol[in] * lam2;
    double tmp = roapf * vol * f_rlencos[iface];
    valcen += -tmp;
    A[c_slot[j * N + i]] = tmp;
  }
  A[c_diag[i]] = valcen;
  bp[i] = bpv;
  dinv[i] = 1.0 / valcen;
}

// BuildPressureMatrix, perfect gas (navier_pressure.cpp:106-224 with DensityModel 1): boundary
// faces of inlets and outlets and the upwind density change enter the rows, which are no longer
// symmetric
__global__ void k_pressure_gas(int ncel, const int* __restrict__ c_nface, const int* __restrict__ c_face,
                               const int* __restrict__ c_slot, const int* __restrict__ c_diag,
                               const int* __restrict__ f_c1, const int* __restrict__ f_c2,
                               const int* __restrict__ f_bnd, const int* __restrict__ b_type,
                               const double* __restrict__ f_lambda, const double* __restrict__ f_rlencos,
                               const double* __restrict__ c_vol, const double* __restrict__ R,
                               const double* __restrict__ T, const double* __restrict__ BRo,
                               const double* __restrict__ Apr, const double* __restrict__ RUFace, int unsteady,
                               double dt, double* __restrict__ A, double* __restrict__ bp, double* __restrict__ dinv) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncel) return;
  const long N = ncel;
  double valcen = 0., bpv = 0.;
  double voli = c_vol[i], Ti = T[i];
  if (unsteady) valcen += -voli / (dt * kRcpcv * Ti);
  int nf = c_nface[i];
  for (int j = 0; j < nf; j++) {
    int iface = c_face[j * N + i];
    int c1 = f_c1[iface], c2 = f_c2[iface];
    bool own = (i == c1);
    if (own) bpv += RUFace[iface];
    else bpv -= RUFace[iface];
    if (c2 < 0) {
      int bnd = f_bnd[iface];
      int t = b_type[bnd];
      double RUn = RUFace[iface];
      if (t == 2) {
        double rof = BRo[bnd];
        valcen += dmin(RUn, 0.) / (rof * kRcpcv * Ti);
      } else if (t == 3) {
        double rof = R[i];
        valcen += (RUn > 0. ? RUn : 0.) / (rof * kRcpcv * Ti);
      }
      continue;
    }
    int in = own ? c2 : c1;
    double lam = own ? f_lambda[iface] : 1. - f_lambda[iface];
    double RUn = own ? RUFace[iface] : -RUFace[iface];
    double lam2 = 1. - lam;
    double roapf = R[i] * Apr[i] * lam + R[in] * Apr[in] * lam2;
    double vol = voli * lam + c_vol[in] * lam2;
    double tmp = roapf * vol * f_rlencos[iface];
    valcen += -tmp;
    double rof = lam * R[i] + lam2 * R[in];
    if (RUn > 0.) {
      double tmp2 = -RUn / (rof * kRcpcv * Ti);
      valcen += tmp2;
    }
    double acn = tmp;
    if (RUn < 0.) acn += -RUn / (rof * kRcpcv * T[in]);
    A[c_slot[j * N + i]] = acn;
  }
  A[c_diag[i]] = valcen;
  bp[i] = bpv;
  dinv[i] = 1.0 / valcen;
}

// pressure, density and velocity correction for a perfect gas (navier_pressure.cpp:45-70,
// DensityModel 1); block partial of localRes[3] as in k_correct_cells
__global__ void k_correct_cells_gas(int ncel, const double* __restrict__ c_vol, const double* __restrict__ dp,
                                    const double* __restrict__ Apr, const double* __restrict__ dPdX,
                                    const double* __restrict__ T, int cell_pref, double urf_p, double* __restrict__ P,
                                    double* __restrict__ R, double* __restrict__ U, double* __restrict__ V,
                                    double* __restrict__ W, double* __restrict__ red) {
  __shared__ double wsum[kThreads / 32];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double r = 0.0;
  if (i < ncel) {
    double ref = dp[cell_pref];
    double vol = c_vol[i];
    r = fabs(dp[i] - ref) * vol;
    P[i] += urf_p * dp[i];
    R[i] += dp[i] / (kRcpcv * T[i]);
    double coef = vol * Apr[i];
    U[i] -= coef * dPdX[3 * (long)i];
    V[i] -= coef * dPdX[3 * (long)i + 1];
    W[i] -= coef * dPdX[3 * (long)i + 2];
  }
  for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = r;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < kThreads / 32; q++) s += wsum[q];
    red[blockIdx.x] = s;
  }
}

// pressure and velocity correction (navier_pressure.cpp:45-70); block partial of
// localRes[3] = sum |p' - p'_ref| * vol
__global__ void k_correct_cells(int ncel, const double* __restrict__ c_vol, const double* __restrict__ dp,
                                const double* __restrict__ Apr, const double* __restrict__ dPdX, int cell_pref,
                                double urf_p, double* __restrict__ P, double* __restrict__ U, double* __restrict__ V,
                                double* __restrict__ W, double* __restrict__ red) {
  __shared__ double wsum[kThreads / 32];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  double r = 0.0;
  if (i < ncel) {
    double ref = dp[cell_pref];
    double d = dp[i] - ref;
    double vol = c_vol[i];
    r = fabs(dp[i] - ref) * vol;
    P[i] += urf_p * d;
    double coef = vol * Apr[i];
    U[i] -= coef * dPdX[3 * (long)i];
    V[i] -= coef * dPdX[3 * (long)i + 1];
    W[i] -= coef * dPdX[3 * (long)i + 2];
  }
  for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = r;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < kThreads / 32; q++) s += wsum[q];
    red[blockIdx.x] = s;
  }
}

// the same correction for a batch: block b takes rows [blk_lo[b], blk_hi[b]) of one case, whose
// reference cell is case_pref[blk_case[b]]; red[b] receives the block's residual
__global__ void k_correct_cells_batch(const int* __restrict__ blk_lo, const int* __restrict__ blk_hi,
                                      const int* __restrict__ blk_case, const int* __restrict__ case_pref,
                                      const double* __restrict__ c_vol, const double* __restrict__ dp,
                                      const double* __restrict__ Apr, const double* __restrict__ dPdX, double urf_p,
                                      double* __restrict__ P, double* __restrict__ U, double* __restrict__ V,
                                      double* __restrict__ W, double* __restrict__ red) {
  __shared__ double wsum[kThreads / 32];
  const int i = blk_lo[blockIdx.x] + threadIdx.x;
  double r = 0.0;
  if (i < blk_hi[blockIdx.x]) {
    double ref = dp[case_pref[blk_case[blockIdx.x]]];
    double d = dp[i] - ref;
    double vol = c_vol[i];
    r = fabs(dp[i] - ref) * vol;
    P[i] += urf_p * d;
    double coef = vol * Apr[i];
    U[i] -= coef * dPdX[3 * (long)i];
    V[i] -= coef * dPdX[3 * (long)i + 1];
    W[i] -= coef * dPdX[3 * (long)i + 2];
  }
  for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = r;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < kThreads / 32; q++) s += wsum[q];
    red[blockIdx.x] = s;
  }
}

// CorrectRUFace2 (navier_pressure.cpp:235-278); T is null for constant density
__global__ void k_correct_ruface(int nfac, const int* __restrict__ f_c1, const int* __restrict__ f_c2,
                                 const int* __restrict__ f_bnd, const double* __restrict__ f_n,
                                 const double* __restrict__ f_lambda, const double* __restrict__ f_rlencos,
                                 const double* __restrict__ f_xpac, const double* __restrict__ f_xnac,
                                 const double* __restrict__ c_x, const double* __restrict__ c_vol,
                                 const double* __restrict__ R, const double* __restrict__ Apr,
                                 const double* __restrict__ dp, const double* __restrict__ dPdX,
                                 const double* __restrict__ BRo, const double* __restrict__ BU,
                                 const double* __restrict__ BV, const double* __restrict__ BW, double urf_p,
                                 const double* __restrict__ T, double* __restrict__ RUFace) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nfac) return;
  int c1 = f_c1[i], c2 = f_c2[i];
  if (c2 < 0) {
    const double* n = f_n + 3 * (long)i;
    int b = f_bnd[i];
    double ro = BRo[b];
    double ruf = BU[b] * ro, rvf = BV[b] * ro, rwf = BW[b] * ro;
    RUFace[i] = ruf * n[0] + rvf * n[1] + rwf * n[2];
    return;
  }
  double lam = f_lambda[i], lam2 = 1. - lam;
  const double* xp = f_xpac + 3 * (long)i;
  const double* xn = f_xnac + 3 * (long)i;
  const double* x1 = c_x + 3 * (long)c1;
  const double* x2 = c_x + 3 * (long)c2;
  if (T) {  // perfect gas: ro' * u
    double rop = dp[c1] / (kRcpcv * T[c1]) * lam + dp[c2] / (kRcpcv * T[c2]) * lam2;
    double rof = R[c1] * lam + R[c2] * lam2;
    double ru = RUFace[i];
    RUFace[i] = ru + ru * rop / rof;
  }
  double roapf = R[c1] * Apr[c1] * lam + R[c2] * Apr[c2] * lam2;
  double vol = c_vol[c1] * lam + c_vol[c2] * lam2;
  double coef = roapf * vol * f_rlencos[i];
  double dp1 = dp[c1] + urf_p * vdot3(dPdX + 3 * (long)c1, xp[0] - x1[0], xp[1] - x1[1], xp[2] - x1[2]);
  double dp2 = dp[c2] + urf_p * vdot3(dPdX + 3 * (long)c2, xn[0] - x2[0], xn[1] - x2[1], xn[2] - x2[2]);
  RUFace[i] += -coef * (dp2 - dp1);
}

// ------------------------------------------------------------------ k-epsilon
// cell sources of UpdateTurKEpsilon (navier_scalar.cpp:33-64)
__global__ void k_keps_sources(int ncel, const double* __restrict__ c_vol, const double* __restrict__ VisLam,
                               const double* __restrict__ VisTur, const double* __restrict__ dU,
                               const double* __restrict__ dV, const double* __restrict__ dW,
                               const double* __restrict__ R, const double* __restrict__ TE,
                               const double* __restrict__ ED, double* VisTE, double* VisED, double* Prod,
                               double* TES, double* ApTE, double* EDS, double* ApED) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncel) return;
  const double Sigma_k = 1.0, Sigma_e = 1.3;
  double vol = c_vol[i];
  VisTE[i] = VisLam[i] + VisTur[i] / Sigma_k;
  VisED[i] = VisLam[i] + VisTur[i] / Sigma_e;
  const double* du = dU + 3 * (long)i;
  const double* dv = dV + 3 * (long)i;
  const double* dw = dW + 3 * (long)i;
  double s1 = (du[0] + du[0]) * du[0] + (du[1] + dv[0]) * du[1] + (du[2] + dw[0]) * du[2];
  double s2 = (dv[0] + du[1]) * dv[0] + (dv[1] + dv[1]) * dv[1] + (dv[2] + dw[1]) * dv[2];
  double s3 = (dw[0] + du[2]) * dw[0] + (dw[1] + dv[2]) * dw[1] + (dw[2] + dw[2]) * dw[2];
  double pr = VisTur[i] * (s1 + s2 + s3);
  Prod[i] = pr;
  double Dis = R[i] * ED[i];
  TES[i] = pr * vol;
  ApTE[i] = Dis / TE[i] * vol;
  EDS[i] = 0.;
  ApED[i] = 0.;
}

// SetBCKEpsilon wall part (navier_bc.cpp:248-286): one thread per wall cell walks that
// cell's wall faces in boundary order, so repeated updates of a corner cell happen in the
// reference's sequence.
// x^1.5 rounded once to nearest, the value pow(x, 1.5) stands for in the wall function
// (navier_bc.cpp:279).  C libraries round pow to within about 0.52 ulp, so their results differ
// from one another and from the exact rounding for a small share of arguments (0.07 % with
// glibc's pow over 1e-9..1e2); the oracle computes the same function as below, so both agree
// to the bit.  x*sqrt(x) with s = sqrt(x) correctly rounded (IEEE), the root's exact remainder
// x - s*s (one FMA) and its Newton correction (x - s*s) / (2s), and the exact error of the
// product x*s (Dekker's two-product by FMA); the sum is within 2^-100 relative of x^1.5 before
// its one rounding.
__device__ __forceinline__ double pow15(double x) {
  if (x == 0.0) return 0.0;
  const double s = sqrt(x);
  const double r = fma(-s, s, x);
  const double d = r / (2.0 * s);
  const double p = x * s;
  const double e = fma(x, s, -p);
  return p + (e + x * d);
}

__global__ void k_keps_wall(int n_wc, const int* __restrict__ wc_cell, const int* __restrict__ wc_start,
                            const int* __restrict__ wc_bnd, const int* __restrict__ b_face,
                            const double* __restrict__ b_dist, const double* __restrict__ f_n,
                            const double* __restrict__ f_area, const double* __restrict__ c_vol,
                            const double* __restrict__ U, const double* __restrict__ V,
                            const double* __restrict__ W, const double* __restrict__ R,
                            const double* __restrict__ VisLam, const double* __restrict__ TE, double* ED,
                            double* BTE, double* BED, double* Prod, double* TES, double* ApTE, double cmu25,
                            double cmu75) {
  int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= n_wc) return;
  const double kappa = 0.419;
  int ic = wc_cell[w];
  double vol = c_vol[ic];
  double u = U[ic], v = V[ic], ww = W[ic], ro = R[ic], mu = VisLam[ic], te = TE[ic];
  double ed = ED[ic], apte = ApTE[ic], prod = Prod[ic], tes = TES[ic];
  for (int q = wc_start[w]; q < wc_start[w + 1]; q++) {
    int i = wc_bnd[q];
    int iface = b_face[i];
    const double* n = f_n + 3 * (long)iface;
    BTE[i] = te;
    BED[i] = ed;
    double ar = f_area[iface];
    double s1 = n[0] / (ar + 1.e-16), s2 = n[1] / (ar + 1.e-16), s3 = n[2] / (ar + 1.e-16);
    double vnor = u * s1 + v * s2 + ww * s3;
    double vt1 = u - vnor * s1, vt2 = v - vnor * s2, vt3 = ww - vnor * s3;
    double vel = sqrt(vt1 * vt1 + vt2 * vt2 + vt3 * vt3);
    double utau = cmu25 * sqrt(te);
    double dist = b_dist[i];
    double yplus = dist * utau * ro / (mu + SMALL);
    double tauw = mu * vel / dist;
    if (yplus < 11.) utau = sqrt(tauw / ro);
    else utau = cmu25 * sqrt(te);
    prod = tauw * utau / (kappa * dist);
    double eps = cmu75 * pow15(te) / (kappa * dist);
    tes = prod * vol;
    apte -= ro * ed / te * vol;
    apte += ro * eps / te * vol;
    ed = eps;
    BED[i] = eps;
  }
  ED[ic] = ed;
  ApTE[ic] = apte;
  Prod[ic] = prod;
  TES[ic] = tes;
}

// SetBCKEpsilon outlet and symmetry copies (navier_bc.cpp:304-326)
__global__ void k_keps_bcopy(int n, const int* __restrict__ lst, const int* __restrict__ b_face,
                             const int* __restrict__ f_c1, const double* __restrict__ TE,
                             const double* __restrict__ ED, double* BTE, double* BED) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  int i = lst[k];
  int ic = f_c1[b_face[i]];
  BTE[i] = TE[ic];
  BED[i] = ED[ic];
}

struct ScaArgs {
  int ncel;
  const int *c_nface, *c_face, *c_slot, *c_diag;
  const int *f_c1, *f_c2, *f_bnd, *b_type;
  const double *f_x, *f_n, *f_lambda, *f_rlencos, *c_x, *RUFace;
  const double *phi, *bphi, *diff, *src, *app0, *dphi;
  double *A, *b, *dinv;
  double urf;
  int* err;
};

// BuildScalarMatrix cell loop (navier_scalar.cpp:421-589), steady
__global__ void __launch_bounds__(kThreads) k_scalar(ScaArgs a) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.ncel) return;
  const long N = a.ncel;
  double phii = a.phi[i], diffi = a.diff[i];
  double xi0 = a.c_x[3 * i], xi1 = a.c_x[3 * i + 1], xi2 = a.c_x[3 * i + 2];
  double gi0 = a.dphi[3 * i], gi1 = a.dphi[3 * i + 1], gi2 = a.dphi[3 * i + 2];
  double app = a.app0[i], sphi = a.src[i];
  int nf = a.c_nface[i];
  for (int j = 0; j < nf; j++) {
    int iface = a.c_face[j * N + i];
    int ip = a.f_c1[iface], in = a.f_c2[iface];
    const double* fn = a.f_n + 3 * (long)iface;
    const double* fx = a.f_x + 3 * (long)iface;
    double fde, fdi, fcs;
    if (in < 0) {
      int bnd = a.f_bnd[iface];
      int t = a.b_type[bnd];
      double RUn = a.RUFace[iface];
      double Visc = diffi;
      double dxc0 = fx[0] - xi0, dxc1 = fx[1] - xi1, dxc2 = fx[2] - xi2;
      double val = Visc * a.f_rlencos[iface];
      app += val;
      fde = Visc * (gi0 * fn[0] + gi1 * fn[1] + gi2 * fn[2]);
      double bp = a.bphi[bnd];
      fdi = val * (gi0 * dxc0 + gi1 * dxc1 + gi2 * dxc2 - bp);
      if (t == 1 || t == 4) {
        fcs = 0.;
      } else {
        if (t == 2 && RUn > 0) atomicOr(a.err, 4);  // the reference stops here
        double fl = dmin(RUn, 0.0);
        app -= fl;
        fcs = fl * bp;
      }
    } else {
      double s1, s2, s3, RUn, lam;
      double fl0 = a.f_lambda[iface];
      if (i != ip) {
        in = ip;
        s1 = -fn[0];
        s2 = -fn[1];
        s3 = -fn[2];
        RUn = -a.RUFace[iface];
        lam = 1. - fl0;
      } else {
        s1 = fn[0];
        s2 = fn[1];
        s3 = fn[2];
        RUn = a.RUFace[iface];
        lam = fl0;
      }
      double lam2 = 1. - lam;
      double gn0 = a.dphi[3 * (long)in], gn1 = a.dphi[3 * (long)in + 1], gn2 = a.dphi[3 * (long)in + 2];
      double Visc = lam * diffi + lam2 * a.diff[in];
      double gx = lam * gi0 + lam2 * gn0, gy = lam * gi1 + lam2 * gn1, gz = lam * gi2 + lam2 * gn2;
      double apn = 0.;
      if (RUn < 0.) {
        apn += RUn;
        app -= RUn;
      }
      double val = Visc * a.f_rlencos[iface];
      app += val;
      apn += -val;
      a.A[a.c_slot[j * N + i]] = apn;
      double phin = a.phi[in];
      double xn0 = a.c_x[3 * (long)in], xn1 = a.c_x[3 * (long)in + 1], xn2 = a.c_x[3 * (long)in + 2];
      double pfi, pfh;
      if (RUn > 0.) {
        pfi = phii;
        pfh = phii + vdot3v(gi0, gi1, gi2, fx[0] - xi0, fx[1] - xi1, fx[2] - xi2);
      } else {
        pfi = phin;
        pfh = phin + vdot3v(gn0, gn1, gn2, fx[0] - xn0, fx[1] - xn1, fx[2] - xn2);
      }
      fcs = RUn * (pfh - pfi);
      fde = Visc * (gx * s1 + gy * s2 + gz * s3);
      fdi = val * (gx * (xn0 - xi0) + gy * (xn1 - xi1) + gz * (xn2 - xi2));
    }
    sphi += fde - fdi - fcs;
  }
  app /= a.urf;
  a.A[a.c_diag[i]] = app;
  a.b[i] = sphi + (1. - a.urf) * app * phii;
  a.dinv[i] = 1.0 / app;
}

// TE clip (navier_scalar.cpp:105-109) fused with the epsilon sources (navier_scalar.cpp:115-121)
__global__ void k_clip_te_eps_sources(int ncel, const double* __restrict__ c_vol, const double* __restrict__ R,
                                      const double* __restrict__ ED, const double* __restrict__ Prod, double* TE,
                                      double* EDS, double* ApED) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncel) return;
  const double Ceps1 = 1.44, Ceps2 = 1.92;
  double te = TE[i];
  if (te < 1.e-9) te = 1.e-9;
  TE[i] = te;
  double fact = ED[i] / (te + SMALL) * c_vol[i];
  EDS[i] = Ceps1 * fact * Prod[i];
  ApED[i] += Ceps2 * fact * R[i];
}

// epsilon rows of wall cells replaced by [1, 0...] with right-hand side ED (navier_scalar.cpp:129-154)
__global__ void k_eps_wall_rows(int n_wc, const int* __restrict__ wc_cell, const int* __restrict__ rowptr,
                                const int* __restrict__ c_diag, const double* __restrict__ ED, double* A, double* b,
                                double* dinv) {
  int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= n_wc) return;
  int ic = wc_cell[w];
  for (int k = rowptr[ic]; k < rowptr[ic + 1]; k++) A[k] = 0.0;
  A[c_diag[ic]] = 1.0;
  b[ic] = ED[ic];
  dinv[ic] = 1.0;
}

// unsteady terms of a scalar equation (navier_scalar.cpp:71-90, 290-305)
__global__ void k_scalar_time(int ncel, const double* __restrict__ c_vol, const double* __restrict__ R, double dt,
                              int scheme, const double* __restrict__ phi_old, double* ap, double* src) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncel) return;
  double coef = R[i] / dt * c_vol[i];
  double po = phi_old[i];
  if (scheme == 1) {
    ap[i] += coef;
    src[i] += coef * po;
  } else {
    ap[i] += 1.5 * coef;
    src[i] += coef * (2 * po - 0.5 * po);
  }
}

// UpdateEnergy diffusion coefficient and sources (navier_scalar.cpp:215-281).  With a perfect
// gas the work of the viscous stresses on each face enters its two cells with opposite signs;
// every cell gathers its faces in ascending face order, the order of the reference's face loop.
__global__ void k_energy_sources(int ncel, int gas, const int* __restrict__ c_nface, const int* __restrict__ c_gface,
                                 const int* __restrict__ f_c1, const int* __restrict__ f_c2,
                                 const double* __restrict__ f_lambda, const double* __restrict__ f_n,
                                 const double* __restrict__ VisLam, const double* __restrict__ VisTur,
                                 const double* __restrict__ dU, const double* __restrict__ dV,
                                 const double* __restrict__ dW, const double* __restrict__ U,
                                 const double* __restrict__ V, const double* __restrict__ W, double* kcond,
                                 double* ES, double* ApE) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncel) return;
  kcond[i] = kCp * (VisLam[i] / kPrl + VisTur[i] / kPrte) / kCp;
  ApE[i] = 0.;
  double es = 0.;
  if (gas) {
    const long N = ncel;
    int nf = c_nface[i];
    for (int j = 0; j < nf; j++) {
      int f = c_gface[j * N + i];
      int c1 = f_c1[f], c2 = f_c2[f];
      double VisL, VisT, g[9], vx, vy, vz;
      if (c2 < 0) {
        VisL = VisLam[c1];
        VisT = VisTur[c1];
        for (int d = 0; d < 3; d++) {
          g[d] = dU[3 * (long)c1 + d];
          g[3 + d] = dV[3 * (long)c1 + d];
          g[6 + d] = dW[3 * (long)c1 + d];
        }
        vx = U[c1];
        vy = V[c1];
        vz = W[c1];
      } else {
        double lam = f_lambda[f], lam2 = 1. - lam;
        VisL = lam * VisLam[c1] + lam2 * VisLam[c2];
        VisT = lam * VisTur[c1] + lam2 * VisTur[c2];
        for (int d = 0; d < 3; d++) {
          g[d] = lam * dU[3 * (long)c1 + d] + lam2 * dU[3 * (long)c2 + d];
          g[3 + d] = lam * dV[3 * (long)c1 + d] + lam2 * dV[3 * (long)c2 + d];
          g[6 + d] = lam * dW[3 * (long)c1 + d] + lam2 * dW[3 * (long)c2 + d];
        }
        vx = lam * U[c1] + lam2 * U[c2];
        vy = lam * V[c1] + lam2 * V[c2];
        vz = lam * W[c1] + lam2 * W[c2];
      }
      double dudx = g[0], dudy = g[1], dudz = g[2], dvdx = g[3], dvdy = g[4], dvdz = g[5];
      double dwdx = g[6], dwdy = g[7], dwdz = g[8];
      double vmul = VisL + VisT;
      double vlac = -2. / 3. * vmul;
      double div = dudx + dvdy + dwdz;
      double txx = 2. * vmul * dudx + vlac * div;
      double tyy = 2. * vmul * dvdy + vlac * div;
      double tzz = 2. * vmul * dwdz + vlac * div;
      double txy = vmul * (dudy + dvdx);
      double txz = vmul * (dudz + dwdx);
      double tyz = vmul * (dvdz + dwdy);
      double btx = vx * txx + vy * txy + vz * txz;
      double bty = vx * txy + vy * tyy + vz * tyz;
      double btz = vx * txz + vy * tyz + vz * tzz;
      const double* n = f_n + 3 * (long)f;
      double fvis = (btx * n[0] + bty * n[1] + btz * n[2]) / kCp;
      if (i == c1) es += fvis;
      else es -= fvis;
    }
  }
  ES[i] = es;
}

// SetBCTemperature (navier_bc.cpp:183-213): outlets and symmetry planes take the cell value;
// walls and inlets keep theirs
__global__ void k_bc_temperature(int nbnd, const int* __restrict__ b_face, const int* __restrict__ b_type,
                                 const int* __restrict__ f_c1, const double* __restrict__ T, double* BTem) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nbnd) return;
  int t = b_type[b];
  if (t == 3 || t == 4) BTem[b] = T[f_c1[b_face[b]]];
}

// epsilon clip and turbulent viscosity (navier_scalar.cpp:165-178)
__global__ void k_finish_keps(int ncel, const double* __restrict__ R, const double* __restrict__ TE, double* ED,
                              double* VisTur) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncel) return;
  const double Cmu = 0.09;
  double ed = ED[i];
  if (ed < 1.e-12) ed = 1.e-12;
  ED[i] = ed;
  VisTur[i] = ed > 1.e-12 ? Cmu * R[i] * TE[i] * TE[i] / (ed + SMALL) : 0.;
}

}  // namespace

// ------------------------------------------------------------------ launch wrappers
void launch_geometry(const DevMesh& m, int* d_err, cudaStream_t s) {
  ++g_launch_count, k_cell_geometry<<<blocks_for(m.ncel), kThreads, 0, s>>>(m.ncel, m.c_vert, m.vert, m.c_vol, m.c_x);
  ++g_launch_count, k_face_geometry<<<blocks_for(m.nfac), kThreads, 0, s>>>(m.nfac, m.f_vert, m.vert, m.f_c1, m.f_c2, m.c_x, m.f_x,
                                                          m.f_n, m.f_area, m.f_lambda, d_err);
  ++g_launch_count, k_face_geometry2<<<blocks_for(m.nfac), kThreads, 0, s>>>(m.nfac, m.f_c1, m.f_c2, m.f_bnd, m.c_x, m.f_x, m.f_n,
                                                           m.f_area, m.f_rlencos, m.f_xpac, m.f_xnac, m.b_dist,
                                                           d_err);
}

void launch_bc_velocity(const DevMesh& m, const DevFields& f, int density_model, bool set_pressure,
                        cudaStream_t s, const DevBatch* b) {
  if (m.nbnd > 0)
    ++g_launch_count, k_bc_velocity<<<blocks_for(m.nbnd), kThreads, 0, s>>>(m.nbnd, m.b_face, m.b_type, m.f_c1, m.f_n, m.f_area, f.R,
                                                          f.U, f.V, f.W, f.P, f.BRo, f.BU, f.BV, f.BW, f.BPre,
                                                          set_pressure ? 1 : 0);
  if (density_model == 0 && m.n_outlet > 0)
    ++g_launch_count, k_bc_outlet<<<b ? b->ncases : 1, kThreads, 0, s>>>(
                          m.n_inlet, m.inlet_list, m.n_outlet, m.outlet_list, m.b_face, m.f_n, m.f_area, f.BRo, f.BU,
                          f.BV, f.BW, b ? b->in0 : nullptr, b ? b->out0 : nullptr);
}

void launch_bc_deltap(const DevMesh& m, const DevFields& f, cudaStream_t s) {
  if (m.nbnd > 0) ++g_launch_count, k_bc_copy<<<blocks_for(m.nbnd), kThreads, 0, s>>>(m.nbnd, m.b_face, m.f_c1, f.dp, f.BPre);
}

template <class T>
void launch_gradient_t(const DevMesh& m, int nfield, const double* const* phi, const double* const* bphi,
                       double* const* grad, cudaStream_t s) {
  if (nfield == 4) {
    GradArgs<4> a;
    for (int q = 0; q < 4; q++) {
      a.phi[q] = phi[q];
      a.bphi[q] = bphi[q];
      a.grad[q] = grad[q];
    }
    ++g_launch_count, k_gradient<T, 4><<<blocks_for(m.ncel), kThreads, 0, s>>>(m.ncel, m.c_nface, m.c_gface, m.f_c1, m.f_c2, m.f_bnd,
                                                          m.f_lambda, m.f_n, m.c_vol, a);
  } else {
    for (int q = 0; q < nfield; q++) {
      GradArgs<1> a;
      a.phi[0] = phi[q];
      a.bphi[0] = bphi[q];
      a.grad[0] = grad[q];
      ++g_launch_count, k_gradient<T, 1><<<blocks_for(m.ncel), kThreads, 0, s>>>(m.ncel, m.c_nface, m.c_gface, m.f_c1, m.f_c2,
                                                            m.f_bnd, m.f_lambda, m.f_n, m.c_vol, a);
    }
  }
}

void launch_gradient(const DevMesh& m, int nfield, const double* const* phi, const double* const* bphi,
                     double* const* grad, cudaStream_t s, bool fp32) {
  if (fp32) launch_gradient_t<float>(m, nfield, phi, bphi, grad, s);
  else launch_gradient_t<double>(m, nfield, phi, bphi, grad, s);
}

void launch_momentum(const DevMesh& m, const DevFields& f, const double* urf, const double* gravity,
                     DevStatus* st, cudaStream_t s, const TimeConf& tc, bool fp32) {
  MomArgs a;
  a.Unp = f.Unp;
  a.Vnp = f.Vnp;
  a.Wnp = f.Wnp;
  a.scheme = tc.scheme;
  a.dt = tc.dt;
  a.ncel = m.ncel;
  a.c_nface = m.c_nface;
  a.c_face = m.c_face;
  a.c_slot = m.c_slot;
  a.c_diag = m.c_diag;
  a.f_c1 = m.f_c1;
  a.f_c2 = m.f_c2;
  a.f_bnd = m.f_bnd;
  a.b_type = m.b_type;
  a.f_x = m.f_x;
  a.f_n = m.f_n;
  a.f_lambda = m.f_lambda;
  a.f_rlencos = m.f_rlencos;
  a.c_x = m.c_x;
  a.c_vol = m.c_vol;
  a.U = f.U;
  a.V = f.V;
  a.W = f.W;
  a.P = f.P;
  a.R = f.R;
  a.VisLam = f.VisLam;
  a.VisTur = f.VisTur;
  a.RUFace = f.RUFace;
  a.dU = f.dUdX;
  a.dV = f.dVdX;
  a.dW = f.dWdX;
  a.dP = f.dPdX;
  a.BU = f.BU;
  a.BV = f.BV;
  a.BW = f.BW;
  a.A = f.Au;
  a.bu = f.bu;
  a.bv = f.bv;
  a.bw = f.bw;
  a.Apr = f.Apr;
  a.dinv = f.dinv_u;
  a.old = f.old;
  a.shear = f.shear;
  a.urf0 = urf[0];
  a.g0 = gravity[0];
  a.g1 = gravity[1];
  a.g2 = gravity[2];
  a.warn = &st->warn_inlet;
  if (fp32) ++g_launch_count, k_momentum<float><<<blocks_for(m.ncel), kThreads, 0, s>>>(a);
  else ++g_launch_count, k_momentum<double><<<blocks_for(m.ncel), kThreads, 0, s>>>(a);
}

void launch_ruface2(const DevMesh& m, const DevFields& f, cudaStream_t s, bool fp32) {
  auto k = fp32 ? k_ruface2<float> : k_ruface2<double>;
  ++g_launch_count, k<<<blocks_for(m.nfac), kThreads, 0, s>>>(m.nfac, m.f_c1, m.f_c2, m.f_bnd, m.f_n, m.f_area, m.f_lambda,
                                            m.f_xpac, m.f_xnac, m.c_x, m.c_vol, f.R, f.U, f.V, f.W, f.P, f.Apr,
                                            f.dPdX, f.BRo, f.BU, f.BV, f.BW, f.RUFace);
}

void launch_pressure(const DevMesh& m, const DevFields& f, cudaStream_t s) {
  ++g_launch_count, k_pressure<<<blocks_for(m.ncel), kThreads, 0, s>>>(m.ncel, m.c_nface, m.c_face, m.c_slot, m.c_diag, m.f_c1,
                                                     m.f_c2, m.f_lambda, m.f_rlencos, m.c_vol, f.R, f.Apr,
                                                     f.RUFace, f.Ap, f.bp, f.dinv_p);
}

void launch_pressure_gas(const DevMesh& m, const DevFields& f, const TimeConf& tc, cudaStream_t s) {
  ++g_launch_count, k_pressure_gas<<<blocks_for(m.ncel), kThreads, 0, s>>>(
                        m.ncel, m.c_nface, m.c_face, m.c_slot, m.c_diag, m.f_c1, m.f_c2, m.f_bnd, m.b_type,
                        m.f_lambda, m.f_rlencos, m.c_vol, f.R, f.T, f.BRo, f.Apr, f.RUFace, tc.scheme != 0 ? 1 : 0,
                        tc.dt, f.Ap, f.bp, f.dinv_p);
}

void launch_correct_cells(const DevMesh& m, const DevFields& f, int cell_pref, double urf_p, double* red,
                          cudaStream_t s, const DevBatch* b, int density_model) {
  if (density_model == 1) {
    ++g_launch_count, k_correct_cells_gas<<<blocks_for(m.ncel), kThreads, 0, s>>>(
                          m.ncel, m.c_vol, f.dp, f.Apr, f.dPdX, f.T, cell_pref, urf_p, f.P, f.R, f.U, f.V, f.W, red);
    return;
  }
  if (b) {
    ++g_launch_count, k_correct_cells_batch<<<b->nblk, kThreads, 0, s>>>(b->blk_lo, b->blk_hi, b->blk_case,
                                                                          b->case_pref, m.c_vol, f.dp, f.Apr, f.dPdX,
                                                                          urf_p, f.P, f.U, f.V, f.W, red);
    return;
  }
  ++g_launch_count, k_correct_cells<<<blocks_for(m.ncel), kThreads, 0, s>>>(m.ncel, m.c_vol, f.dp, f.Apr, f.dPdX, cell_pref, urf_p,
                                                          f.P, f.U, f.V, f.W, red);
}

void launch_correct_ruface(const DevMesh& m, const DevFields& f, double urf_p, cudaStream_t s, int density_model) {
  ++g_launch_count, k_correct_ruface<<<blocks_for(m.nfac), kThreads, 0, s>>>(m.nfac, m.f_c1, m.f_c2, m.f_bnd, m.f_n, m.f_lambda,
                                                           m.f_rlencos, m.f_xpac, m.f_xnac, m.c_x, m.c_vol, f.R,
                                                           f.Apr, f.dp, f.dPdX, f.BRo, f.BU, f.BV, f.BW, urf_p,
                                                           density_model == 1 ? f.T : nullptr, f.RUFace);
}

void launch_scalar_time(const DevMesh& m, const DevFields& f, const TimeConf& tc, const double* phi_old, double* ap,
                        double* src, cudaStream_t s) {
  ++g_launch_count, k_scalar_time<<<blocks_for(m.ncel), kThreads, 0, s>>>(m.ncel, m.c_vol, f.R, tc.dt, tc.scheme,
                                                                          phi_old, ap, src);
}

void launch_energy_sources(const DevMesh& m, const DevFields& f, int density_model, cudaStream_t s) {
  ++g_launch_count, k_energy_sources<<<blocks_for(m.ncel), kThreads, 0, s>>>(
                        m.ncel, density_model == 1 ? 1 : 0, m.c_nface, m.c_gface, m.f_c1, m.f_c2, m.f_lambda, m.f_n,
                        f.VisLam, f.VisTur, f.dUdX, f.dVdX, f.dWdX, f.U, f.V, f.W, f.kcond, f.ES, f.ApE);
}

void launch_bc_temperature(const DevMesh& m, const DevFields& f, cudaStream_t s) {
  if (m.nbnd > 0)
    ++g_launch_count, k_bc_temperature<<<blocks_for(m.nbnd), kThreads, 0, s>>>(m.nbnd, m.b_face, m.b_type, m.f_c1, f.T,
                                                                               f.BTem);
}

void launch_keps_sources(const DevMesh& m, const DevFields& f, cudaStream_t s) {
  ++g_launch_count, k_keps_sources<<<blocks_for(m.ncel), kThreads, 0, s>>>(m.ncel, m.c_vol, f.VisLam, f.VisTur, f.dUdX, f.dVdX,
                                                         f.dWdX, f.R, f.TE, f.ED, f.VisTE, f.VisED, f.Prod, f.TES,
                                                         f.ApTE, f.EDS, f.ApED);
}

void launch_keps_wall(const DevMesh& m, const DevFields& f, cudaStream_t s) {
  // Cmu^0.25 and Cmu^0.75 are constants of the model; evaluated once on the host with the
  // same pow the reference calls.
  static const double cmu25 = __builtin_pow(0.09, 0.25);
  static const double cmu75 = __builtin_pow(0.09, 0.75);
  if (m.n_wallcell > 0)
    ++g_launch_count, k_keps_wall<<<blocks_for(m.n_wallcell), kThreads, 0, s>>>(m.n_wallcell, m.wc_cell, m.wc_start, m.wc_bnd,
                                                              m.b_face, m.b_dist, m.f_n, m.f_area, m.c_vol, f.U, f.V,
                                                              f.W, f.R, f.VisLam, f.TE, f.ED, f.BTE, f.BED, f.Prod,
                                                              f.TES, f.ApTE, cmu25, cmu75);
  if (m.n_outlet > 0)
    ++g_launch_count, k_keps_bcopy<<<blocks_for(m.n_outlet), kThreads, 0, s>>>(m.n_outlet, m.outlet_list, m.b_face, m.f_c1, f.TE,
                                                             f.ED, f.BTE, f.BED);
  if (m.n_sym > 0)
    ++g_launch_count, k_keps_bcopy<<<blocks_for(m.n_sym), kThreads, 0, s>>>(m.n_sym, m.sym_list, m.b_face, m.f_c1, f.TE, f.ED,
                                                          f.BTE, f.BED);
}

void launch_scalar(const DevMesh& m, const DevFields& f, const double* phi, const double* bphi, const double* diff,
                   const double* src, const double* app, double urf_s, DevStatus* st, cudaStream_t s) {
  ScaArgs a;
  a.ncel = m.ncel;
  a.c_nface = m.c_nface;
  a.c_face = m.c_face;
  a.c_slot = m.c_slot;
  a.c_diag = m.c_diag;
  a.f_c1 = m.f_c1;
  a.f_c2 = m.f_c2;
  a.f_bnd = m.f_bnd;
  a.b_type = m.b_type;
  a.f_x = m.f_x;
  a.f_n = m.f_n;
  a.f_lambda = m.f_lambda;
  a.f_rlencos = m.f_rlencos;
  a.c_x = m.c_x;
  a.RUFace = f.RUFace;
  a.phi = phi;
  a.bphi = bphi;
  a.diff = diff;
  a.src = src;
  a.app0 = app;
  a.dphi = f.dPhidX;
  a.A = f.As;
  a.b = f.bs;
  a.dinv = f.dinv_s;
  a.urf = urf_s;
  a.err = &st->err;
  ++g_launch_count, k_scalar<<<blocks_for(m.ncel), kThreads, 0, s>>>(a);
}

void launch_clip_te(const DevMesh& m, const DevFields& f, cudaStream_t s) {
  ++g_launch_count, k_clip_te_eps_sources<<<blocks_for(m.ncel), kThreads, 0, s>>>(m.ncel, m.c_vol, f.R, f.ED, f.Prod, f.TE, f.EDS,
                                                                f.ApED);
}

void launch_eps_wall_rows(const DevMesh& m, const DevFields& f, cudaStream_t s) {
  if (m.n_wallcell > 0)
    ++g_launch_count, k_eps_wall_rows<<<blocks_for(m.n_wallcell), kThreads, 0, s>>>(m.n_wallcell, m.wc_cell, m.rowptr, m.c_diag,
                                                                  f.ED, f.As, f.bs, f.dinv_s);
}

void launch_finish_keps(const DevMesh& m, const DevFields& f, cudaStream_t s) {
  ++g_launch_count, k_finish_keps<<<blocks_for(m.ncel), kThreads, 0, s>>>(m.ncel, f.R, f.TE, f.ED, f.VisTur);
}

}  // namespace cycas
