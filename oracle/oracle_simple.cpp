// CPU ORACLE — TEST INFRASTRUCTURE ONLY (see oracle.h; parity unpinned at the PETSc boundary).
// One SIMPLE iteration of NavierStokesSolver::NSSolve restated at one rank (steady or one outer
// iteration of a transient step; constant density or perfect gas; k-epsilon; energy).
#include <algorithm>
#include <cmath>
#include <stdexcept>

#include "oracle.h"

namespace orc {

static inline void vminus(double* a, const double* b, const double* c) {
  for (int i = 0; i < 3; i++) a[i] = b[i] - c[i];
}
static inline double vdot(const double* a, const double* b) {
  double s = 0.;
  for (int i = 0; i < 3; i++) s += a[i] * b[i];
  return s;
}
static inline double vlen(const double* a) {
  double s = 0.;
  for (int i = 0; i < 3; i++) s += a[i] * a[i];
  return std::sqrt(s);
}
static inline double dmin(double x, double y) { return x < y ? x : y; }  // CYCASMIN, tools.h:12

static int type1Of(Case& cs, int rid) {
  auto it = cs.regionMap.find(rid);
  if (it == cs.regionMap.end()) throw std::runtime_error("unknown region id");
  return it->second.type1;
}

// SetBCVelocity (navier_bc.cpp:8-119)
void set_bc_velocity(Case& cs) {
  for (int i = 0; i < cs.Nbnd; i++) {
    int iface = cs.B[i].face, ic = cs.F[iface].cell1;
    switch (type1Of(cs, cs.B[i].rid)) {
      case 1:
        cs.BRo[i] = cs.Rn[ic];
        cs.BU[i] = 0.;
        cs.BV[i] = 0.;
        cs.BW[i] = 0.;
        break;
      case 2:
        break;
      case 3:
        cs.BRo[i] = cs.Rn[ic];
        cs.BU[i] = cs.Un[ic];
        cs.BV[i] = cs.Vn[ic];
        cs.BW[i] = cs.Wn[ic];
        break;
      case 4: {
        const Face& f = cs.F[iface];
        double s1 = f.n[0] / f.area, s2 = f.n[1] / f.area, s3 = f.n[2] / f.area;
        double un = cs.Un[ic] * s1 + cs.Vn[ic] * s2 + cs.Wn[ic] * s3;
        cs.BU[i] = cs.Un[ic] - un * s1;
        cs.BV[i] = cs.Vn[ic] - un * s2;
        cs.BW[i] = cs.Wn[ic] - un * s3;
        cs.BRo[i] = cs.Rn[ic];
        break;
      }
      default:
        throw std::runtime_error("no such boundary type in velocity bc");
    }
  }
  if (cs.DensityModel == 0) {
    double min = 0.0, mout = 0.0, aout = 0.0;
    for (int i = 0; i < cs.Nbnd; i++) {
      int iface = cs.B[i].face;
      const double* n = cs.F[iface].n;
      int t = type1Of(cs, cs.B[i].rid);
      if (t == 2)
        min += cs.BRo[i] * (cs.BU[i] * n[0] + cs.BV[i] * n[1] + cs.BW[i] * n[2]);
      else if (t == 3) {
        mout += cs.BRo[i] * (cs.BU[i] * n[0] + cs.BV[i] * n[1] + cs.BW[i] * n[2]);
        aout += cs.BRo[i] * cs.F[i].area;  // Face[i] with the boundary index, as the reference writes it
      }
    }
    // MPI_Allreduce over one rank is the identity
    if (std::fabs(mout) > SMALL) {
      double rate = -min / mout;
      for (int i = 0; i < cs.Nbnd; i++) {
        int iface = cs.B[i].face;  // BU[iface]: boundary faces come first, iface == i
        if (type1Of(cs, cs.B[i].rid) == 3) {
          cs.BU[iface] *= rate;
          cs.BV[iface] *= rate;
          cs.BW[iface] *= rate;
        }
      }
    } else {
      double rate = (-min - mout) / aout;
      for (int i = 0; i < cs.Nbnd; i++) {
        int iface = cs.B[i].face;
        if (type1Of(cs, cs.B[i].rid) == 3) {
          const Face& f = cs.F[iface];
          cs.BU[iface] += rate * f.n[0] / f.area;
          cs.BV[iface] += rate * f.n[1] / f.area;
          cs.BW[iface] += rate * f.n[2] / f.area;
        }
      }
    }
  }
}

// SetBCPressure (navier_bc.cpp:121-155): every non-periodic type copies the cell value
void set_bc_pressure(Case& cs) {
  for (int i = 0; i < cs.Nbnd; i++) {
    int ic = cs.F[cs.B[i].face].cell1;
    int t = type1Of(cs, cs.B[i].rid);
    if (t >= 1 && t <= 4) cs.BPre[i] = cs.Pn[ic];
    else throw std::runtime_error("no such boundary type");
  }
}

// SetBCDeltaP (navier_bc.cpp:157-181)
void set_bc_deltap(Case& cs) {
  for (int i = 0; i < cs.Nbnd; i++) {
    int ic = cs.F[cs.B[i].face].cell1;
    int t = type1Of(cs, cs.B[i].rid);
    if (t >= 1 && t <= 4) cs.BPre[i] = cs.deltaP[ic];
    else throw std::runtime_error("no such boundary type");
  }
}

// Gradient (navier_gradient.cpp:12-74), limiter 0
void gradient(Case& cs, const double* phi, const double* Bphif, double* g) {
  for (int i = 0; i < 3 * cs.Ncel; i++) g[i] = 0.;
  for (int i = 0; i < cs.Nfac; i++) {
    const Face& f = cs.F[i];
    int c1 = f.cell1, c2 = f.cell2;
    if (c2 >= 0) {
      double pf = f.lambda * phi[c1] + (1. - f.lambda) * phi[c2];
      for (int d = 0; d < 3; d++) {
        g[3 * c1 + d] += pf * f.n[d];
        g[3 * c2 + d] -= pf * f.n[d];
      }
    } else {
      double pf = Bphif[f.bnd];
      for (int d = 0; d < 3; d++) g[3 * c1 + d] += pf * f.n[d];
    }
  }
  for (int i = 0; i < cs.Ncel; i++)
    for (int d = 0; d < 3; d++) g[3 * i + d] /= cs.C[i].vol;
}

// BuildVelocityMatrix (navier_velocity.cpp:63-393)
void build_velocity_matrix(Case& cs) {
  set_bc_velocity(cs);
  set_bc_pressure(cs);
  gradient(cs, cs.Un.data(), cs.BU.data(), cs.dUdX.data());
  gradient(cs, cs.Vn.data(), cs.BV.data(), cs.dVdX.data());
  gradient(cs, cs.Wn.data(), cs.BW.data(), cs.dWdX.data());
  gradient(cs, cs.Pn.data(), cs.BPre.data(), cs.dPdX.data());
  const double* dU = cs.dUdX.data();
  const double* dV = cs.dVdX.data();
  const double* dW = cs.dWdX.data();
  for (int i = 0; i < cs.Ncel; i++) {
    const Cell& ci = cs.C[i];
    double app = 0., su = 0., sv = 0., sw = 0., apn[6] = {0, 0, 0, 0, 0, 0};
    int ani[6], nj = 0;
    double fcs[3] = {0., 0., 0.}, fde[3], fdi[3];
    if (!cs.IfSteady) {  // unsteady terms (navier_velocity.cpp:108-123)
      if (cs.TimeScheme == 1) {
        double coef = cs.Rn[i] / cs.dt * ci.vol;
        app += coef;
        su += coef * cs.Unp[i];
        sv += coef * cs.Vnp[i];
        sw += coef * cs.Wnp[i];
      } else if (cs.TimeScheme == 2) {
        double coef = cs.Rn[i] / cs.dt * ci.vol;
        app += 1.5 * coef;
        su += coef * (2 * cs.Unp[i] - 0.5 * cs.Unp2[i]);
        sv += coef * (2 * cs.Vnp[i] - 0.5 * cs.Vnp2[i]);
        sw += coef * (2 * cs.Wnp[i] - 0.5 * cs.Wnp2[i]);
      }
    }
    for (int j = 0; j < ci.nface; j++) {
      int iface = ci.face[j];
      const Face& f = cs.F[iface];
      int ip = f.cell1, in = f.cell2;
      if (in < 0) {
        int bnd = f.bnd;
        int t = type1Of(cs, cs.B[bnd].rid);
        double s1 = f.n[0], s2 = f.n[1], s3 = f.n[2];
        double RUnormal = cs.RUFace[iface];
        double Visc = cs.VisLam[i] + cs.VisTur[i];
        double dudx = dU[3 * i], dudy = dU[3 * i + 1], dudz = dU[3 * i + 2];
        double dvdx = dV[3 * i], dvdy = dV[3 * i + 1], dvdz = dV[3 * i + 2];
        double dwdx = dW[3 * i], dwdy = dW[3 * i + 1], dwdz = dW[3 * i + 2];
        double dxc[3];
        vminus(dxc, f.x, ci.x);
        double val;
        switch (t) {
          case 1: {
            val = Visc * f.rlencos;
            app += val;
            Bnd& b = cs.B[bnd];
            b.shear[0] = (dudx + dudx) * s1 + (dudy + dvdx) * s2 + (dudz + dwdx) * s3;
            b.shear[1] = (dvdx + dudy) * s1 + (dvdy + dvdy) * s2 + (dvdz + dwdy) * s3;
            b.shear[2] = (dwdx + dudz) * s1 + (dwdy + dvdz) * s2 + (dwdz + dwdz) * s3;
            for (int d = 0; d < 3; d++) b.shear[d] *= Visc;
            b.shear[0] += cs.Pn[i] * s1;
            b.shear[1] += cs.Pn[i] * s2;
            b.shear[2] += cs.Pn[i] * s3;
            fde[0] = val * cs.Un[i];
            fde[1] = val * cs.Vn[i];
            fde[2] = val * cs.Wn[i];
            fdi[0] = val * cs.Un[i];
            fdi[1] = val * cs.Vn[i];
            fdi[2] = val * cs.Wn[i];
            break;
          }
          case 2:
          case 3:
          case 4:
            val = Visc * f.rlencos;
            app += val;
            fde[0] = (dudx + dudx) * s1 + (dudy + dvdx) * s2 + (dudz + dwdx) * s3;
            fde[1] = (dvdx + dudy) * s1 + (dvdy + dvdy) * s2 + (dvdz + dwdy) * s3;
            fde[2] = (dwdx + dudz) * s1 + (dwdy + dvdz) * s2 + (dwdz + dwdz) * s3;
            fde[0] *= Visc;
            fde[1] *= Visc;
            fde[2] *= Visc;
            fdi[0] = val * (dudx * dxc[0] + dudy * dxc[1] + dudz * dxc[2] - cs.BU[bnd]);
            fdi[1] = val * (dvdx * dxc[0] + dvdy * dxc[1] + dvdz * dxc[2] - cs.BV[bnd]);
            fdi[2] = val * (dwdx * dxc[0] + dwdy * dxc[1] + dwdz * dxc[2] - cs.BW[bnd]);
            break;
          default:
            throw std::runtime_error("no such rid");
        }
        switch (t) {
          case 1:
          case 4:
            fcs[0] = fcs[1] = fcs[2] = 0.;
            break;
          case 2:
          case 3: {
            if (t == 2 && RUnormal > 0) cs.reverseInletWarnings++;
            double fl = dmin(RUnormal, 0.0);
            app -= fl;
            fcs[0] = fl * cs.BU[bnd];
            fcs[1] = fl * cs.BV[bnd];
            fcs[2] = fl * cs.BW[bnd];
            break;
          }
        }
      } else {
        double s1, s2, s3, RUnormal, lambda;
        if (i != ip) {
          in = ip;
          s1 = -f.n[0];
          s2 = -f.n[1];
          s3 = -f.n[2];
          RUnormal = -cs.RUFace[iface];
          lambda = 1. - f.lambda;
        } else {
          s1 = f.n[0];
          s2 = f.n[1];
          s3 = f.n[2];
          RUnormal = cs.RUFace[iface];
          lambda = f.lambda;
        }
        double lambda2 = 1. - lambda;
        double Visc = lambda * (cs.VisLam[i] + cs.VisTur[i]) + lambda2 * (cs.VisLam[in] + cs.VisTur[in]);
        double dudx = lambda * dU[3 * i] + lambda2 * dU[3 * in];
        double dudy = lambda * dU[3 * i + 1] + lambda2 * dU[3 * in + 1];
        double dudz = lambda * dU[3 * i + 2] + lambda2 * dU[3 * in + 2];
        double dvdx = lambda * dV[3 * i] + lambda2 * dV[3 * in];
        double dvdy = lambda * dV[3 * i + 1] + lambda2 * dV[3 * in + 1];
        double dvdz = lambda * dV[3 * i + 2] + lambda2 * dV[3 * in + 2];
        double dwdx = lambda * dW[3 * i] + lambda2 * dW[3 * in];
        double dwdy = lambda * dW[3 * i + 1] + lambda2 * dW[3 * in + 1];
        double dwdz = lambda * dW[3 * i + 2] + lambda2 * dW[3 * in + 2];
        if (RUnormal < 0.) {
          apn[nj] += RUnormal;
          app -= RUnormal;
        }
        double val = Visc * f.rlencos;
        app += val;
        apn[nj] += -val;
        ani[nj] = cs.C[in].globalIdx;
        nj++;
        double ufi, vfi, wfi, ufh, vfh, wfh, dx[3];
        if (RUnormal > 0.) {
          ufi = cs.Un[i];
          vfi = cs.Vn[i];
          wfi = cs.Wn[i];
          vminus(dx, f.x, ci.x);
          ufh = cs.Un[i] + vdot(dU + 3 * i, dx);
          vfh = cs.Vn[i] + vdot(dV + 3 * i, dx);
          wfh = cs.Wn[i] + vdot(dW + 3 * i, dx);
        } else {
          ufi = cs.Un[in];
          vfi = cs.Vn[in];
          wfi = cs.Wn[in];
          vminus(dx, f.x, cs.C[in].x);
          ufh = cs.Un[in] + vdot(dU + 3 * in, dx);
          vfh = cs.Vn[in] + vdot(dV + 3 * in, dx);
          wfh = cs.Wn[in] + vdot(dW + 3 * in, dx);
        }
        fcs[0] = RUnormal * (ufh - ufi);
        fcs[1] = RUnormal * (vfh - vfi);
        fcs[2] = RUnormal * (wfh - wfi);
        fde[0] = (dudx + dudx) * s1 + (dudy + dvdx) * s2 + (dudz + dwdx) * s3;
        fde[1] = (dvdx + dudy) * s1 + (dvdy + dvdy) * s2 + (dvdz + dwdy) * s3;
        fde[2] = (dwdx + dudz) * s1 + (dwdy + dvdz) * s2 + (dwdz + dwdz) * s3;
        fde[0] *= Visc;
        fde[1] *= Visc;
        fde[2] *= Visc;
        double dxc[3];
        vminus(dxc, cs.C[in].x, ci.x);
        fdi[0] = val * (dudx * dxc[0] + dudy * dxc[1] + dudz * dxc[2]);
        fdi[1] = val * (dvdx * dxc[0] + dvdy * dxc[1] + dvdz * dxc[2]);
        fdi[2] = val * (dwdx * dxc[0] + dwdy * dxc[1] + dwdz * dxc[2]);
      }
      su += fde[0] - fdi[0] - fcs[0];
      sv += fde[1] - fdi[1] - fcs[1];
      sw += fde[2] - fdi[2] - fcs[2];
    }
    app /= cs.URF[0];
    cs.Apr[i] = 1. / (app);
    int row = ci.globalIdx;
    cs.Au.insert(row, row, app);
    for (int k = 0; k < nj; k++) cs.Au.insert(row, ani[k], apn[k]);
    double vol = ci.vol;
    cs.bu[row] = su + (1. - cs.URF[0]) * app * cs.Un[i] + (-cs.dPdX[3 * i] + cs.Rn[i] * cs.gravity[0]) * vol;
    cs.bv[row] = sv + (1. - cs.URF[0]) * app * cs.Vn[i] + (-cs.dPdX[3 * i + 1] + cs.Rn[i] * cs.gravity[1]) * vol;
    cs.bw[row] = sw + (1. - cs.URF[0]) * app * cs.Wn[i] + (-cs.dPdX[3 * i + 2] + cs.Rn[i] * cs.gravity[2]) * vol;
  }
}

// CalRUFace2, Rhie-Chow interpolation (navier_velocity.cpp:425-477)
void cal_ruface2(Case& cs) {
  for (int i = 0; i < cs.Nfac; i++) {
    const Face& f = cs.F[i];
    int c1 = f.cell1, c2 = f.cell2;
    if (c2 < 0) {
      int bnd = f.bnd;
      double ruf = cs.BU[bnd] * cs.BRo[bnd], rvf = cs.BV[bnd] * cs.BRo[bnd], rwf = cs.BW[bnd] * cs.BRo[bnd];
      cs.RUFace[i] = ruf * f.n[0] + rvf * f.n[1] + rwf * f.n[2];
    } else {
      double lambda = f.lambda, lambda2 = 1. - lambda;
      double rf = lambda * cs.Rn[c1] + lambda2 * cs.Rn[c2];
      double ruf = lambda * cs.Rn[c1] * cs.Un[c1] + lambda2 * cs.Rn[c2] * cs.Un[c2];
      double rvf = lambda * cs.Rn[c1] * cs.Vn[c1] + lambda2 * cs.Rn[c2] * cs.Vn[c2];
      double rwf = lambda * cs.Rn[c1] * cs.Wn[c1] + lambda2 * cs.Rn[c2] * cs.Wn[c2];
      cs.RUFace[i] = ruf * f.n[0] + rvf * f.n[1] + rwf * f.n[2];
      double dx[3];
      vminus(dx, f.Xpac, cs.C[c1].x);
      double P1 = cs.Pn[c1] + vdot(&cs.dPdX[3 * c1], dx);
      vminus(dx, f.Xnac, cs.C[c2].x);
      double P2 = cs.Pn[c2] + vdot(&cs.dPdX[3 * c2], dx);
      vminus(dx, f.Xnac, f.Xpac);
      double d12 = vlen(dx);
      double aprf = lambda * cs.Apr[c1] + lambda2 * cs.Apr[c2];
      double vol = lambda * cs.C[c1].vol + lambda2 * cs.C[c2].vol;
      double dpx = lambda * cs.dPdX[3 * c1] + lambda2 * cs.dPdX[3 * c2];
      double dpy = lambda * cs.dPdX[3 * c1 + 1] + lambda2 * cs.dPdX[3 * c2 + 1];
      double dpz = lambda * cs.dPdX[3 * c1 + 2] + lambda2 * cs.dPdX[3 * c2 + 2];
      double dpn = dpx * dx[0] + dpy * dx[1] + dpz * dx[2];
      cs.RUFace[i] -= rf * f.area * aprf / d12 * vol * ((P2 - P1) - dpn);
    }
  }
}

// BuildPressureMatrix (navier_pressure.cpp:99-232)
void build_pressure_matrix(Case& cs) {
  if (cs.DensityModel != 0 && cs.DensityModel != 1) throw std::runtime_error("unknown DensityModel found");
  const bool gas = cs.DensityModel == 1;
  for (int i = 0; i < cs.Ncel; i++) {
    const Cell& ci = cs.C[i];
    double valcen = 0., bpv = 0., Acn[7];
    int cn[7], nj = 0;
    if (!cs.IfSteady && gas) valcen += -ci.vol / (cs.dt * cs.Rcpcv * cs.Tn[i]);
    for (int j = 0; j < ci.nface; j++) {
      int iface = ci.face[j];
      const Face& f = cs.F[iface];
      if (i == f.cell1) bpv += cs.RUFace[iface];
      else bpv -= cs.RUFace[iface];
      int in = ci.cell[j];
      if (in < 0) {
        if (!gas) continue;
        int bnd = f.bnd;
        int t = type1Of(cs, cs.B[bnd].rid);
        double RUnormal = cs.RUFace[iface];
        if (t == 2) {  // inlet
          double rof = cs.BRo[bnd], Tf = cs.Tn[i];
          valcen += dmin(RUnormal, 0.) / (rof * cs.Rcpcv * Tf);
        } else if (t == 3) {  // outlet
          double rof = cs.Rn[i], Tf = cs.Tn[i];
          valcen += (RUnormal > 0. ? RUnormal : 0.) / (rof * cs.Rcpcv * Tf);  // CYCASMAX
        }
        continue;
      }
      double lambda, RUnormal;
      if (i == f.cell1) {
        lambda = f.lambda;
        RUnormal = cs.RUFace[iface];
      } else {
        lambda = 1. - f.lambda;
        RUnormal = -cs.RUFace[iface];
      }
      double lambda2 = 1. - lambda;
      double roapf = cs.Rn[i] * cs.Apr[i] * lambda + cs.Rn[in] * cs.Apr[in] * lambda2;
      double vol = ci.vol * lambda + cs.C[in].vol * lambda2;
      double tmp = roapf * vol * f.rlencos;
      valcen += -tmp;
      if (!gas) {
        Acn[nj] = tmp;
      } else {
        double rof = lambda * cs.Rn[i] + lambda2 * cs.Rn[in];
        if (RUnormal > 0.) {
          double Tf = cs.Tn[i];
          double tmp2 = -RUnormal / (rof * cs.Rcpcv * Tf);
          valcen += tmp2;
        }
        Acn[nj] = tmp;
        if (RUnormal < 0.) {
          double Tf = cs.Tn[in];
          Acn[nj] += -RUnormal / (rof * cs.Rcpcv * Tf);
        }
      }
      cn[nj] = cs.C[in].globalIdx;
      nj++;
    }
    int row = ci.globalIdx;
    cs.Ap.insert(row, row, valcen);
    for (int k = 0; k < nj; k++) cs.Ap.insert(row, cn[k], Acn[k]);
    cs.bp[row] = bpv;
  }
}

// pressure (and density) and velocity correction (navier_pressure.cpp:45-70)
void correct_cells(Case& cs) {
  double ref = cs.deltaP[cs.cellPressureRef];  // root rank value; MPI_Bcast at one rank is the identity
  for (int i = 0; i < cs.Ncel; i++) {
    cs.localRes[3] += std::fabs(cs.deltaP[i] - ref) * cs.C[i].vol;
    if (cs.DensityModel == 0) {
      cs.Pn[i] += cs.URF[3] * (cs.deltaP[i] - ref);
    } else if (cs.DensityModel == 1) {  // perfect gas
      cs.Pn[i] += cs.URF[3] * cs.deltaP[i];
      cs.Rn[i] += cs.deltaP[i] / (cs.Rcpcv * cs.Tn[i]);
    }
    double coef = cs.C[i].vol * cs.Apr[i];
    cs.Un[i] -= coef * cs.dPdX[3 * i];
    cs.Vn[i] -= coef * cs.dPdX[3 * i + 1];
    cs.Wn[i] -= coef * cs.dPdX[3 * i + 2];
  }
}

// CorrectRUFace2 (navier_pressure.cpp:235-278)
void correct_ruface2(Case& cs) {
  const double* dp = cs.deltaP.data();
  for (int i = 0; i < cs.Nfac; i++) {
    const Face& f = cs.F[i];
    int c1 = f.cell1, c2 = f.cell2;
    if (c2 < 0) {
      int bnd = f.bnd;
      double ruf = cs.BU[bnd] * cs.BRo[bnd], rvf = cs.BV[bnd] * cs.BRo[bnd], rwf = cs.BW[bnd] * cs.BRo[bnd];
      cs.RUFace[i] = ruf * f.n[0] + rvf * f.n[1] + rwf * f.n[2];
      continue;
    }
    double lambda = f.lambda, lambda2 = 1. - lambda, dx1[3], dx2[3];
    vminus(dx1, f.Xpac, cs.C[c1].x);
    vminus(dx2, f.Xnac, cs.C[c2].x);
    if (cs.DensityModel == 1) {  // ro'*u
      double rop = dp[c1] / (cs.Rcpcv * cs.Tn[c1]) * lambda + dp[c2] / (cs.Rcpcv * cs.Tn[c2]) * lambda2;
      double rof = cs.Rn[c1] * lambda + cs.Rn[c2] * lambda2;
      cs.RUFace[i] += cs.RUFace[i] * rop / rof;
    }
    double roapf = cs.Rn[c1] * cs.Apr[c1] * lambda + cs.Rn[c2] * cs.Apr[c2] * lambda2;
    double vol = cs.C[c1].vol * lambda + cs.C[c2].vol * lambda2;
    double coef = roapf * vol * f.rlencos;
    double dp1 = dp[c1] + cs.URF[3] * vdot(&cs.dPdX[3 * c1], dx1);
    double dp2 = dp[c2] + cs.URF[3] * vdot(&cs.dPdX[3 * c2], dx2);
    cs.RUFace[i] += -coef * (dp2 - dp1);
  }
}

static void solve_or_throw(Case& cs, const Csr& A, int which, double tol, int maxit, bool guess_zero,
                           const double* b, double* x, const char* name, int force_type = -1) {
  KspSettings s = cs.ksp[which];
  if (force_type >= 0) s.type = force_type;
  double rtol = s.rtol_override > 0 ? s.rtol_override : tol;
  int mi = s.maxit_override > 0 ? s.maxit_override : maxit;
  KspResult r = ksp_solve(A, s, rtol, mi, guess_zero, b, x);
  cs.kspLog.push_back(r);
  if (r.reason < 0) {
    cs.kspFailures++;
    throw std::runtime_error(std::string(name) + " not converge in iter: " + std::to_string(r.its));
  }
}

// CalculateVelocity (navier_velocity.cpp:10-60)
int calculate_velocity(Case& cs) {
  build_velocity_matrix(cs);
  std::vector<double> u0(cs.Un), v0(cs.Vn), w0(cs.Wn);
  solve_or_throw(cs, cs.Au, 0, 1.e-8, 1000, false, cs.bu.data(), cs.Un.data(), "Un");
  solve_or_throw(cs, cs.Au, 0, 1.e-8, 1000, false, cs.bv.data(), cs.Vn.data(), "Vn");
  solve_or_throw(cs, cs.Au, 0, 1.e-8, 1000, false, cs.bw.data(), cs.Wn.data(), "Wn");
  cs.Au.zero();
  for (int i = 0; i < cs.Ncel; i++) {
    cs.localRes[0] += std::fabs(u0[i] - cs.Un[i]) * cs.C[i].vol;
    cs.localRes[1] += std::fabs(v0[i] - cs.Vn[i]) * cs.C[i].vol;
    cs.localRes[2] += std::fabs(w0[i] - cs.Wn[i]) * cs.C[i].vol;
  }
  return 0;
}

// CalculatePressure (navier_pressure.cpp:9-97)
int calculate_pressure(Case& cs) {
  set_bc_velocity(cs);
  cal_ruface2(cs);
  build_pressure_matrix(cs);
  // CG for the symmetric constant-density system, GMRES otherwise (MPIStructure.cpp:462-467)
  solve_or_throw(cs, cs.Ap, 1, 1.e-6, 1000, true, cs.bp.data(), cs.deltaP.data(), "Pn",
                 cs.DensityModel == 0 ? -1 : (int)KSP_GMRES);
  cs.Ap.zero();
  set_bc_deltap(cs);
  gradient(cs, cs.deltaP.data(), cs.BPre.data(), cs.dPdX.data());
  correct_cells(cs);
  set_bc_velocity(cs);
  correct_ruface2(cs);
  return 0;
}

// BuildScalarMatrix (navier_scalar.cpp:407-592)
void build_scalar_matrix(Case& cs, int iSca, double* Phi, double* BPhi, double* DiffCoef, double* source, double* App) {
  (void)iSca;
  double* dP = cs.dPhidX.data();
  gradient(cs, Phi, BPhi, dP);
  for (int i = 0; i < cs.Ncel; i++) {
    const Cell& ci = cs.C[i];
    double app = App[i], sphi = source[i], apn[6] = {0, 0, 0, 0, 0, 0};
    int ani[6], nj = 0;
    double fcs = 0., fde = 0., fdi = 0.;
    for (int j = 0; j < ci.nface; j++) {
      int iface = ci.face[j];
      const Face& f = cs.F[iface];
      int ip = f.cell1, in = f.cell2;
      if (in < 0) {
        int bnd = f.bnd;
        int t = type1Of(cs, cs.B[bnd].rid);
        double s1 = f.n[0], s2 = f.n[1], s3 = f.n[2];
        double RUnormal = cs.RUFace[iface];
        double Visc = DiffCoef[i];
        double gx = dP[3 * i], gy = dP[3 * i + 1], gz = dP[3 * i + 2];
        double dxc[3];
        vminus(dxc, f.x, ci.x);
        if (t < 1 || t > 4) throw std::runtime_error("no such bid");
        double val = Visc * f.rlencos;
        app += val;
        fde = Visc * (gx * s1 + gy * s2 + gz * s3);
        fdi = val * (gx * dxc[0] + gy * dxc[1] + gz * dxc[2] - BPhi[bnd]);
        if (t == 1 || t == 4) {
          fcs = 0.;
        } else {
          if (t == 2 && RUnormal > 0) throw std::runtime_error("reverse flow get out of inlet. stop!");
          double fl = dmin(RUnormal, 0.0);
          app -= fl;
          fcs = fl * BPhi[bnd];
        }
      } else {
        double s1, s2, s3, RUnormal, lambda;
        if (i != ip) {
          in = ip;
          s1 = -f.n[0];
          s2 = -f.n[1];
          s3 = -f.n[2];
          RUnormal = -cs.RUFace[iface];
          lambda = 1. - f.lambda;
        } else {
          s1 = f.n[0];
          s2 = f.n[1];
          s3 = f.n[2];
          RUnormal = cs.RUFace[iface];
          lambda = f.lambda;
        }
        double lambda2 = 1. - lambda;
        double Visc = lambda * DiffCoef[i] + lambda2 * DiffCoef[in];
        double gx = lambda * dP[3 * i] + lambda2 * dP[3 * in];
        double gy = lambda * dP[3 * i + 1] + lambda2 * dP[3 * in + 1];
        double gz = lambda * dP[3 * i + 2] + lambda2 * dP[3 * in + 2];
        if (RUnormal < 0.) {
          apn[nj] += RUnormal;
          app -= RUnormal;
        }
        double val = Visc * f.rlencos;
        app += val;
        apn[nj] += -val;
        ani[nj] = cs.C[in].globalIdx;
        nj++;
        double pfi, pfh, dx[3];
        if (RUnormal > 0.) {
          pfi = Phi[i];
          vminus(dx, f.x, ci.x);
          pfh = Phi[i] + vdot(dP + 3 * i, dx);
        } else {
          pfi = Phi[in];
          vminus(dx, f.x, cs.C[in].x);
          pfh = Phi[in] + vdot(dP + 3 * in, dx);
        }
        fcs = RUnormal * (pfh - pfi);
        fde = Visc * (gx * s1 + gy * s2 + gz * s3);
        double dxc[3];
        vminus(dxc, cs.C[in].x, ci.x);
        fdi = val * (gx * dxc[0] + gy * dxc[1] + gz * dxc[2]);
      }
      sphi += fde - fdi - fcs;
    }
    app /= cs.URF[5];
    int row = ci.globalIdx;
    cs.As.insert(row, row, app);
    for (int k = 0; k < nj; k++) cs.As.insert(row, ani[k], apn[k]);
    cs.bs[row] = sphi + (1. - cs.URF[5]) * app * Phi[i];
  }
}

// UpdateTurKEpsilon (navier_scalar.cpp:11-197) with SetBCKEpsilon (navier_bc.cpp:220-345)
namespace {
const double kKappa = 0.419, kCmuKE = 0.09, kCeps1 = 1.44, kCeps2 = 1.92, kSigmaK = 1.0, kSigmaE = 1.3;

// TE^1.5 of the wall function (navier_bc.cpp:279, std::pow there), rounded once to nearest.
// The C library's pow is within about 0.52 ulp and misrounds a small share of arguments (0.07 %
// over 1e-9..1e2 with glibc), differently from one library to the next; this restatement takes
// the mathematical value instead, which the GPU computes the same way: x*sqrt(x) with the
// correctly rounded root s, its exact remainder x - s*s, the Newton correction
// (x - s*s) / (2s), and the exact error of x*s (Dekker's two-product by FMA).
double pow15(double x) {
  if (x == 0.0) return 0.0;
  const double s = std::sqrt(x);
  const double r = std::fma(-s, s, x);
  const double d = r / (2.0 * s);
  const double p = x * s;
  const double e = std::fma(x, s, -p);
  return p + (e + x * d);
}
}

// UpdateTurKEpsilon (navier_scalar.cpp:11-197): k rows
void keps_build_te(Case& cs) {
  const double kappa = kKappa, Cmu = kCmuKE, Sigma_k = kSigmaK, Sigma_e = kSigmaE;
  int n = cs.Ncel;
  cs.Prod.assign(n, 0.0);
  cs.TESource.assign(n, 0.0);
  cs.EDSource.assign(n, 0.0);
  cs.ApTE.assign(n, 0.0);
  cs.ApED.assign(n, 0.0);
  cs.VisTE.assign(n, 0.0);
  cs.VisED.assign(n, 0.0);
  std::vector<double>& VisTE = cs.VisTE;
  std::vector<double>& VisED = cs.VisED;
  double *Prod = cs.Prod.data(), *TES = cs.TESource.data(), *EDS = cs.EDSource.data();
  double *ApTE = cs.ApTE.data(), *ApED = cs.ApED.data();
  for (int i = 0; i < n; i++) {
    double vol = cs.C[i].vol;
    VisTE[i] = cs.VisLam[i] + cs.VisTur[i] / Sigma_k;
    VisED[i] = cs.VisLam[i] + cs.VisTur[i] / Sigma_e;
    const double* du = &cs.dUdX[3 * i];
    const double* dv = &cs.dVdX[3 * i];
    const double* dw = &cs.dWdX[3 * i];
    double s1 = (du[0] + du[0]) * du[0] + (du[1] + dv[0]) * du[1] + (du[2] + dw[0]) * du[2];
    double s2 = (dv[0] + du[1]) * dv[0] + (dv[1] + dv[1]) * dv[1] + (dv[2] + dw[1]) * dv[2];
    double s3 = (dw[0] + du[2]) * dw[0] + (dw[1] + dv[2]) * dw[1] + (dw[2] + dw[2]) * dw[2];
    Prod[i] = cs.VisTur[i] * (s1 + s2 + s3);
    double Dis = cs.Rn[i] * cs.ED[i];
    TES[i] = Prod[i] * vol;
    ApTE[i] = Dis / cs.TE[i] * vol;
  }
  // SetBCKEpsilon: wall faces in boundary order, then outlets, then symmetry planes
  for (int i = 0; i < cs.Nbnd; i++) {
    int iface = cs.B[i].face, ic = cs.F[iface].cell1;
    if (type1Of(cs, cs.B[i].rid) != 1) continue;
    const Face& f = cs.F[iface];
    cs.BTE[i] = cs.TE[ic];
    cs.BED[i] = cs.ED[ic];
    double vol = cs.C[ic].vol;
    double s1 = f.n[0] / (f.area + 1.e-16), s2 = f.n[1] / (f.area + 1.e-16), s3 = f.n[2] / (f.area + 1.e-16);
    double vnor = cs.Un[ic] * s1 + cs.Vn[ic] * s2 + cs.Wn[ic] * s3;
    double vt1 = cs.Un[ic] - vnor * s1, vt2 = cs.Vn[ic] - vnor * s2, vt3 = cs.Wn[ic] - vnor * s3;
    double vel = std::sqrt(vt1 * vt1 + vt2 * vt2 + vt3 * vt3);
    double Cmu25 = std::pow(Cmu, 0.25);
    double utau = Cmu25 * std::sqrt(cs.TE[ic]);
    double dist = cs.B[i].distance;
    double yplus = dist * utau * cs.Rn[ic] / (cs.VisLam[ic] + SMALL);
    double tauw = cs.VisLam[ic] * vel / dist;
    if (yplus < 11.) utau = std::sqrt(tauw / cs.Rn[ic]);
    else utau = Cmu25 * std::sqrt(cs.TE[ic]);
    Prod[ic] = tauw * utau / (kappa * dist);
    double te15 = cs.libm_pow ? std::pow(cs.TE[ic], 1.5) : pow15(cs.TE[ic]);
    double eps = std::pow(Cmu, 0.75) * te15 / (kappa * dist);
    TES[ic] = Prod[ic] * vol;
    ApTE[ic] -= cs.Rn[ic] * cs.ED[ic] / cs.TE[ic] * vol;
    ApTE[ic] += cs.Rn[ic] * eps / cs.TE[ic] * vol;
    cs.ED[ic] = eps;
    cs.BED[i] = eps;
  }
  for (int pass = 3; pass <= 4; pass++)
    for (int i = 0; i < cs.Nbnd; i++) {
      int ic = cs.F[cs.B[i].face].cell1;
      if (type1Of(cs, cs.B[i].rid) != pass) continue;
      cs.BTE[i] = cs.TE[ic];
      cs.BED[i] = cs.ED[ic];
    }

  if (!cs.IfSteady) {  // unsteady terms (navier_scalar.cpp:71-90)
    for (int i = 0; i < n; i++) {
      double coef = cs.Rn[i] / cs.dt * cs.C[i].vol;
      if (cs.TimeScheme == 1) {
        ApTE[i] += coef;
        TES[i] += coef * cs.TEp[i];
        ApED[i] += coef;
        EDS[i] += coef * cs.EDp[i];
      } else if (cs.TimeScheme == 2) {
        ApTE[i] += 1.5 * coef;
        TES[i] += coef * (2 * cs.TEp[i] - 0.5 * cs.TEp2[i]);
        ApED[i] += 1.5 * coef;
        EDS[i] += coef * (2 * cs.EDp[i] - 0.5 * cs.EDp2[i]);
      }
    }
  }
  build_scalar_matrix(cs, 2, cs.TE.data(), cs.BTE.data(), VisTE.data(), TES, ApTE);
}

// epsilon rows on the solved k
void keps_build_ed(Case& cs) {
  const double Ceps1 = kCeps1, Ceps2 = kCeps2;
  int n = cs.Ncel;
  double *Prod = cs.Prod.data(), *EDS = cs.EDSource.data(), *ApED = cs.ApED.data();
  cs.As.zero();
  for (int i = 0; i < n; i++)
    if (cs.TE[i] < 1.e-9) cs.TE[i] = 1.e-9;
  for (int i = 0; i < n; i++) {
    double fact = cs.ED[i] / (cs.TE[i] + SMALL) * cs.C[i].vol;
    EDS[i] = Ceps1 * fact * Prod[i];
    ApED[i] += Ceps2 * fact * cs.Rn[i];
  }
  build_scalar_matrix(cs, 3, cs.ED.data(), cs.BED.data(), cs.VisED.data(), EDS, ApED);
  for (int i = 0; i < cs.Nbnd; i++) {
    if (type1Of(cs, cs.B[i].rid) != 1) continue;
    int ic = cs.F[cs.B[i].face].cell1;
    const Cell& c = cs.C[ic];
    int row = c.globalIdx;
    cs.As.insert(row, row, 1.0);
    for (int j = 0; j < c.nface; j++) {
      int icn = c.cell[j];
      if (icn == VOID_CELL_ON_BOUNDARY) continue;
      cs.As.insert(row, cs.C[icn].globalIdx, 0.0);
    }
    cs.bs[row] = cs.ED[ic];
  }
}

void update_tur_kepsilon(Case& cs) {
  const double Cmu = kCmuKE;
  const int n = cs.Ncel;
  keps_build_te(cs);
  solve_or_throw(cs, cs.As, 2, 1.e-8, 500, false, cs.bs.data(), cs.TE.data(), "Tn");
  keps_build_ed(cs);
  solve_or_throw(cs, cs.As, 2, 1.e-8, 500, false, cs.bs.data(), cs.ED.data(), "ED");
  cs.As.zero();
  for (int i = 0; i < n; i++)
    if (cs.ED[i] < 1.e-12) cs.ED[i] = 1.e-12;
  for (int i = 0; i < n; i++) {
    if (cs.ED[i] > 1.e-12) cs.VisTur[i] = Cmu * cs.Rn[i] * cs.TE[i] * cs.TE[i] / (cs.ED[i] + SMALL);
    else cs.VisTur[i] = 0.;
  }
}

// SetBCTemperature (navier_bc.cpp:183-213): walls and inlets keep their values
void set_bc_temperature(Case& cs) {
  for (int i = 0; i < cs.Nbnd; i++) {
    int ic = cs.F[cs.B[i].face].cell1;
    int t = type1Of(cs, cs.B[i].rid);
    if (t == 3 || t == 4) cs.BTem[i] = cs.Tn[ic];
    else if (t != 1 && t != 2) throw std::runtime_error("no such boundary type");
  }
}

// UpdateEnergy (navier_scalar.cpp:204-326) up to the assembled system (As, bs)
void build_energy(Case& cs) {
  const int n = cs.Ncel;
  cs.kcond.assign(n, 0.0);
  cs.ESource.assign(n, 0.0);
  cs.ApE.assign(n, 0.0);
  double *kcond = cs.kcond.data(), *ES = cs.ESource.data(), *ApE = cs.ApE.data();
  for (int i = 0; i < n; i++) kcond[i] = cs.cp * (cs.VisLam[i] / cs.prl + cs.VisTur[i] / cs.prte) / cs.cp;
  if (cs.DensityModel == 1) {  // work of the viscous stresses, face by face
    const double* dU = cs.dUdX.data();
    const double* dV = cs.dVdX.data();
    const double* dW = cs.dWdX.data();
    for (int i = 0; i < cs.Nfac; i++) {
      const Face& f = cs.F[i];
      int c1 = f.cell1, c2 = f.cell2;
      double VisL, VisT, dudx, dudy, dudz, dvdx, dvdy, dvdz, dwdx, dwdy, dwdz, vxg, vyg, vzg;
      if (c2 < 0) {
        VisL = cs.VisLam[c1];
        VisT = cs.VisTur[c1];
        dudx = dU[3 * c1]; dudy = dU[3 * c1 + 1]; dudz = dU[3 * c1 + 2];
        dvdx = dV[3 * c1]; dvdy = dV[3 * c1 + 1]; dvdz = dV[3 * c1 + 2];
        dwdx = dW[3 * c1]; dwdy = dW[3 * c1 + 1]; dwdz = dW[3 * c1 + 2];
        vxg = cs.Un[c1];
        vyg = cs.Vn[c1];
        vzg = cs.Wn[c1];
      } else {
        double lambda = f.lambda, lambda2 = 1. - lambda;
        VisL = lambda * cs.VisLam[c1] + lambda2 * cs.VisLam[c2];
        VisT = lambda * cs.VisTur[c1] + lambda2 * cs.VisTur[c2];
        dudx = lambda * dU[3 * c1] + lambda2 * dU[3 * c2];
        dudy = lambda * dU[3 * c1 + 1] + lambda2 * dU[3 * c2 + 1];
        dudz = lambda * dU[3 * c1 + 2] + lambda2 * dU[3 * c2 + 2];
        dvdx = lambda * dV[3 * c1] + lambda2 * dV[3 * c2];
        dvdy = lambda * dV[3 * c1 + 1] + lambda2 * dV[3 * c2 + 1];
        dvdz = lambda * dV[3 * c1 + 2] + lambda2 * dV[3 * c2 + 2];
        dwdx = lambda * dW[3 * c1] + lambda2 * dW[3 * c2];
        dwdy = lambda * dW[3 * c1 + 1] + lambda2 * dW[3 * c2 + 1];
        dwdz = lambda * dW[3 * c1 + 2] + lambda2 * dW[3 * c2 + 2];
        vxg = lambda * cs.Un[c1] + lambda2 * cs.Un[c2];
        vyg = lambda * cs.Vn[c1] + lambda2 * cs.Vn[c2];
        vzg = lambda * cs.Wn[c1] + lambda2 * cs.Wn[c2];
      }
      double vmul = VisL + VisT;
      double vlac = -2. / 3. * vmul;
      double div = dudx + dvdy + dwdz;
      double txx = 2. * vmul * dudx + vlac * div;
      double tyy = 2. * vmul * dvdy + vlac * div;
      double tzz = 2. * vmul * dwdz + vlac * div;
      double txy = vmul * (dudy + dvdx);
      double txz = vmul * (dudz + dwdx);
      double tyz = vmul * (dvdz + dwdy);
      double btx = vxg * txx + vyg * txy + vzg * txz;
      double bty = vxg * txy + vyg * tyy + vzg * tyz;
      double btz = vxg * txz + vyg * tyz + vzg * tzz;
      double fvis = (btx * f.n[0] + bty * f.n[1] + btz * f.n[2]) / cs.cp;
      ES[c1] += fvis;
      if (c2 >= 0) ES[c2] -= fvis;
    }
  }
  set_bc_temperature(cs);
  if (!cs.IfSteady) {
    for (int i = 0; i < n; i++) {
      double coef = cs.Rn[i] / cs.dt * cs.C[i].vol;
      if (cs.TimeScheme == 1) {
        ApE[i] += coef;
        ES[i] += coef * cs.Tnp[i];
      } else if (cs.TimeScheme == 2) {
        ApE[i] += 1.5 * coef;
        ES[i] += coef * (2 * cs.Tnp[i] - 0.5 * cs.Tnp2[i]);
      }
    }
  }
  build_scalar_matrix(cs, 1, cs.Tn.data(), cs.BTem.data(), kcond, ES, ApE);
}

void update_energy(Case& cs) {
  build_energy(cs);
  solve_or_throw(cs, cs.As, 2, 1.e-8, 500, false, cs.bs.data(), cs.Tn.data(), "Energy");
  cs.As.zero();
}

// SaveTransientOldData (navier.cpp:698-740).  The second-order branch assigns both previous
// levels from the current one (Unp2 = Unp = Un), so the two levels are always equal.
void save_transient_old_data(Case& cs) {
  const int n = cs.Ncel;
  const bool ke = cs.TurModel == 1;
  if (cs.TimeScheme == 1) {
    for (int i = 0; i < n; i++) {
      cs.Rnp[i] = cs.Rn[i];
      cs.Unp[i] = cs.Un[i];
      cs.Vnp[i] = cs.Vn[i];
      cs.Wnp[i] = cs.Wn[i];
      cs.Tnp[i] = cs.Tn[i];
      if (ke) {
        cs.TEp[i] = cs.TE[i];
        cs.EDp[i] = cs.ED[i];
      }
    }
  } else if (cs.TimeScheme == 2) {
    for (int i = 0; i < n; i++) {
      cs.Rnp2[i] = cs.Rnp[i] = cs.Rn[i];
      cs.Unp2[i] = cs.Unp[i] = cs.Un[i];
      cs.Vnp2[i] = cs.Vnp[i] = cs.Vn[i];
      cs.Wnp2[i] = cs.Wnp[i] = cs.Wn[i];
      cs.Tnp2[i] = cs.Tnp[i] = cs.Tn[i];
      if (ke) {
        cs.TEp2[i] = cs.TEp[i] = cs.TE[i];
        cs.EDp2[i] = cs.EDp[i] = cs.ED[i];
      }
    }
  } else {
    throw std::runtime_error("No unsteady time advance scheme");
  }
}

int time_step(Case& cs, std::vector<double>* resmax, std::vector<double>* residuals, std::vector<KspResult>* ksp) {
  if (cs.IfSteady) throw std::runtime_error("time_step needs a transient case");
  save_transient_old_data(cs);
  cs.cur_time += cs.dt;
  double ResMax0 = 0.;
  int iter;
  for (iter = 1; iter < cs.MaxOuterStep; iter++) {
    double ResMax = simple_iteration(cs);
    if (resmax) resmax->push_back(ResMax);
    if (residuals) residuals->insert(residuals->end(), cs.Residual, cs.Residual + RESIDUAL_LEN);
    if (ksp) {
      for (int k = 0; k < 8; k++) ksp->push_back(k < (int)cs.kspLog.size() ? cs.kspLog[k] : KspResult{-1, -1, 0});
    }
    if (iter == 1) ResMax0 = ResMax;
    if (ResMax0 / (ResMax + 1.e-16) > 100.) break;
  }
  return iter < cs.MaxOuterStep ? iter : std::max(0, cs.MaxOuterStep - 1);
}

// one pass of the outer loop (navier.cpp:60-111)
double simple_iteration(Case& cs) {
  std::fill(cs.localRes, cs.localRes + RESIDUAL_LEN, 0.0);
  std::fill(cs.Residual, cs.Residual + RESIDUAL_LEN, 0.0);
  cs.kspLog.clear();
  calculate_velocity(cs);
  calculate_pressure(cs);
  if (cs.TurModel == 1) update_tur_kepsilon(cs);
  if (cs.SolveEnergy) update_energy(cs);
  for (int i = 0; i < RESIDUAL_LEN; i++) cs.Residual[i] = cs.localRes[i];
  double s = 0.;
  for (int i = 0; i < RESIDUAL_LEN; i++) s = s > cs.Residual[i] ? s : cs.Residual[i];  // vec_max, tools.cpp:45-51
  cs.step++;
  return s;
}

}  // namespace orc
