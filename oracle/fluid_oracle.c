/* CPU restatement of the reference's fluid stencils (fluid.F90:2-249 and the
 * fluid halo fill of boundary.F90:122-247), test infrastructure only: the
 * parity reference for the GPU fluid kernels and their timed CPU baseline.
 *
 * Each statement is restated with the reference's operations in the
 * reference's order (gfortran -O3 on x86-64 without -march: left-to-right,
 * no FMA contraction; this file is built with -ffp-contract=off).  Parity
 * pinned: every field each stencil writes agrees bit for bit with the
 * reference's own subroutines run through tests/golden/fortran_subset.py
 * (tests/test_reference_pins.py::test_fluid_stencils_match_the_reference).
 *
 * One rank: the MPI exchanges of FillGhostRegionForFluid become the periodic
 * copies and wall mirrors of DealWithBoundaryFluid, face by face in the
 * reference's order, and ModifyBulkVelocity's MPI_REDUCE of one rank is its
 * local sum (SUM over the interior in array order, one accumulator). */
#include "ibmdem_oracle.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define FHALO 2 /* lap (vars.F90:14) */

struct orc_fluid {
  int n[3], ni, nj, nk;
  int SG[3], EG[3], LG[3], UG[3];
  int64_t ncell;
  int bType[6];
  double dx, dy, dz, dt, rhof;
  double visc, CPx, CPy, CPz;
  double *f[IBMDEM_FLUID_NFIELDS];
};

static inline int64_t fx_(const orc_fluid* F, int i, int j, int k) {
  return ((int64_t)(k - F->LG[2]) * F->nj + (j - F->LG[1])) * F->ni + (i - F->LG[0]);
}

orc_fluid* orc_fluid_create(const ibmdem_params* p) {
  orc_fluid* F = (orc_fluid*)calloc(1, sizeof(orc_fluid));
  if (!F) return NULL;
  F->n[0] = p->nx;
  F->n[1] = p->ny;
  F->n[2] = p->nz;
  for (int d = 0; d < 3; ++d) {
    F->SG[d] = 1;
    F->EG[d] = F->n[d];
    F->LG[d] = 1 - FHALO;
    F->UG[d] = F->n[d] + FHALO;
  }
  F->ni = F->n[0] + 2 * FHALO;
  F->nj = F->n[1] + 2 * FHALO;
  F->nk = F->n[2] + 2 * FHALO;
  F->ncell = (int64_t)F->ni * F->nj * F->nk;
  for (int s = 0; s < 6; ++s) F->bType[s] = p->bType[s];
  F->dx = p->dx;
  F->dy = p->dy;
  F->dz = p->dz;
  F->dt = p->dt;
  F->rhof = p->rhof;
  for (int q = 0; q < IBMDEM_FLUID_NFIELDS; ++q) {
    F->f[q] = (double*)calloc((size_t)F->ncell, sizeof(double));
    if (!F->f[q]) {
      orc_fluid_destroy(F);
      return NULL;
    }
  }
  return F;
}

void orc_fluid_destroy(orc_fluid* F) {
  if (!F) return;
  for (int q = 0; q < IBMDEM_FLUID_NFIELDS; ++q) free(F->f[q]);
  free(F);
}

void orc_fluid_set_params(orc_fluid* F, double visc, double CPx, double CPy, double CPz) {
  F->visc = visc;
  F->CPx = CPx;
  F->CPy = CPy;
  F->CPz = CPz;
}

int orc_fluid_set_field(orc_fluid* F, int which, const double* a) {
  if (which < 0 || which >= IBMDEM_FLUID_NFIELDS || !a) return IBMDEM_EINVAL;
  memcpy(F->f[which], a, sizeof(double) * (size_t)F->ncell);
  return 0;
}

int orc_fluid_get_field(orc_fluid* F, int which, double* a) {
  if (which < 0 || which >= IBMDEM_FLUID_NFIELDS || !a) return IBMDEM_EINVAL;
  memcpy(a, F->f[which], sizeof(double) * (size_t)F->ncell);
  return 0;
}

#define U F->f[IBMDEM_FLUID_U]
#define V F->f[IBMDEM_FLUID_V]
#define W F->f[IBMDEM_FLUID_W]
#define LOOP_INTERIOR                       \
  for (int k = F->SG[2]; k <= F->EG[2]; ++k) \
    for (int j = F->SG[1]; j <= F->EG[1]; ++j) \
      for (int i = F->SG[0]; i <= F->EG[0]; ++i)

/* uold = u; vold = v; wold = w (fluid.F90:257) */
void orc_fluid_StoreOldVelocity(orc_fluid* F) {
  memcpy(F->f[IBMDEM_FLUID_UOLD], U, sizeof(double) * (size_t)F->ncell);
  memcpy(F->f[IBMDEM_FLUID_VOLD], V, sizeof(double) * (size_t)F->ncell);
  memcpy(F->f[IBMDEM_FLUID_WOLD], W, sizeof(double) * (size_t)F->ncell);
}

/* VelocityGuess (fluid.F90:108-133) with ConvectionTensor (fluid.F90:2-54),
 * ViscousTensor (fluid.F90:56-76) and PressureGradient (fluid.F90:78-91): the
 * tensors of every interior node are formed from u,v,w as they stand, then
 * u,v,w take uold + dt*(a*RHS + b*RHSl - c*grad P) and RHSl takes RHS. */
void orc_fluid_VelocityGuess(orc_fluid* F, double aRK, double bRK, double cRK) {
  const double dx = F->dx, dy = F->dy, dz = F->dz, dt = F->dt, rhof = F->rhof, visc = F->visc;
  const double CPx = F->CPx, CPy = F->CPy, CPz = F->CPz;
  const double *u = U, *v = V, *w = W, *P = F->f[IBMDEM_FLUID_P];
  const double *fx = F->f[IBMDEM_FLUID_FX], *fy = F->f[IBMDEM_FLUID_FY], *fz = F->f[IBMDEM_FLUID_FZ];
  double* nu = (double*)malloc(sizeof(double) * 3 * (size_t)F->ncell);
  if (!nu) return;
  double *nv = nu + F->ncell, *nw = nv + F->ncell;
#pragma omp parallel for schedule(static)
  for (int k = F->SG[2]; k <= F->EG[2]; ++k)
    for (int j = F->SG[1]; j <= F->EG[1]; ++j)
      for (int i = F->SG[0]; i <= F->EG[0]; ++i) {
#define A(f, a, b, c) f[fx_(F, a, b, c)]
        const double uuE = 0.5 * (A(u, i + 1, j, k) + A(u, i, j, k)) * 0.5 * (A(u, i + 1, j, k) + A(u, i, j, k));
        const double uuW = 0.5 * (A(u, i - 1, j, k) + A(u, i, j, k)) * 0.5 * (A(u, i - 1, j, k) + A(u, i, j, k));
        const double uvB = 0.5 * (A(u, i, j + 1, k) + A(u, i, j, k)) * 0.5 * (A(v, i - 1, j + 1, k) + A(v, i, j + 1, k));
        const double uvF = 0.5 * (A(u, i, j - 1, k) + A(u, i, j, k)) * 0.5 * (A(v, i - 1, j, k) + A(v, i, j, k));
        const double uwN = 0.5 * (A(u, i, j, k + 1) + A(u, i, j, k)) * 0.5 * (A(w, i - 1, j, k + 1) + A(w, i, j, k + 1));
        const double uwS = 0.5 * (A(u, i, j, k - 1) + A(u, i, j, k)) * 0.5 * (A(w, i - 1, j, k) + A(w, i, j, k));

        const double vuE = 0.5 * (A(v, i + 1, j, k) + A(v, i, j, k)) * 0.5 * (A(u, i + 1, j - 1, k) + A(u, i + 1, j, k));
        const double vuW = 0.5 * (A(v, i - 1, j, k) + A(v, i, j, k)) * 0.5 * (A(u, i, j - 1, k) + A(u, i, j, k));
        const double vvB = 0.5 * (A(v, i, j + 1, k) + A(v, i, j, k)) * 0.5 * (A(v, i, j + 1, k) + A(v, i, j, k));
        const double vvF = 0.5 * (A(v, i, j - 1, k) + A(v, i, j, k)) * 0.5 * (A(v, i, j - 1, k) + A(v, i, j, k));
        const double vwN = 0.5 * (A(v, i, j, k + 1) + A(v, i, j, k)) * 0.5 * (A(w, i, j - 1, k + 1) + A(w, i, j, k + 1));
        const double vwS = 0.5 * (A(v, i, j, k - 1) + A(v, i, j, k)) * 0.5 * (A(w, i, j - 1, k) + A(w, i, j, k));

        const double wuE = 0.5 * (A(w, i + 1, j, k) + A(w, i, j, k)) * 0.5 * (A(u, i + 1, j, k - 1) + A(u, i + 1, j, k));
        const double wuW = 0.5 * (A(w, i - 1, j, k) + A(w, i, j, k)) * 0.5 * (A(u, i, j, k - 1) + A(u, i, j, k));
        const double wvB = 0.5 * (A(w, i, j + 1, k) + A(w, i, j, k)) * 0.5 * (A(v, i, j + 1, k - 1) + A(v, i, j + 1, k));
        const double wvF = 0.5 * (A(w, i, j - 1, k) + A(w, i, j, k)) * 0.5 * (A(v, i, j, k - 1) + A(v, i, j, k));
        const double wwN = 0.5 * (A(w, i, j, k + 1) + A(w, i, j, k)) * 0.5 * (A(w, i, j, k + 1) + A(w, i, j, k));
        const double wwS = 0.5 * (A(w, i, j, k - 1) + A(w, i, j, k)) * 0.5 * (A(w, i, j, k - 1) + A(w, i, j, k));

        const double TIux = (uuE - uuW) / dx, TIuy = (uvB - uvF) / dy, TIuz = (uwN - uwS) / dz;
        const double TIvx = (vuE - vuW) / dx, TIvy = (vvB - vvF) / dy, TIvz = (vwN - vwS) / dz;
        const double TIwx = (wuE - wuW) / dx, TIwy = (wvB - wvF) / dy, TIwz = (wwN - wwS) / dz;

        /* 2*u(i,j,k): the integer 2 becomes 2.0d0 */
        const double TVux = (A(u, i + 1, j, k) + A(u, i - 1, j, k) - 2 * A(u, i, j, k)) / (dx * dx) * visc;
        const double TVuy = (A(u, i, j + 1, k) + A(u, i, j - 1, k) - 2 * A(u, i, j, k)) / (dy * dy) * visc;
        const double TVuz = (A(u, i, j, k + 1) + A(u, i, j, k - 1) - 2 * A(u, i, j, k)) / (dz * dz) * visc;
        const double TVvx = (A(v, i + 1, j, k) + A(v, i - 1, j, k) - 2 * A(v, i, j, k)) / (dx * dx) * visc;
        const double TVvy = (A(v, i, j + 1, k) + A(v, i, j - 1, k) - 2 * A(v, i, j, k)) / (dy * dy) * visc;
        const double TVvz = (A(v, i, j, k + 1) + A(v, i, j, k - 1) - 2 * A(v, i, j, k)) / (dz * dz) * visc;
        const double TVwx = (A(w, i + 1, j, k) + A(w, i - 1, j, k) - 2 * A(w, i, j, k)) / (dx * dx) * visc;
        const double TVwy = (A(w, i, j + 1, k) + A(w, i, j - 1, k) - 2 * A(w, i, j, k)) / (dy * dy) * visc;
        const double TVwz = (A(w, i, j, k + 1) + A(w, i, j, k - 1) - 2 * A(w, i, j, k)) / (dz * dz) * visc;

        const double Px = (A(P, i, j, k) - A(P, i - 1, j, k)) / (dx) / rhof;
        const double Py = (A(P, i, j, k) - A(P, i, j - 1, k)) / (dy) / rhof;
        const double Pz = (A(P, i, j, k) - A(P, i, j, k - 1)) / (dz) / rhof;
#undef A
        const int64_t c = fx_(F, i, j, k);
        const double RHSu = -(TIux + TIuy + TIuz) + (TVux + TVuy + TVuz) + CPx + fx[c];
        const double RHSv = -(TIvx + TIvy + TIvz) + (TVvx + TVvy + TVvz) + CPy + fy[c];
        const double RHSw = -(TIwx + TIwy + TIwz) + (TVwx + TVwy + TVwz) + CPz + fz[c];
        nu[c] = F->f[IBMDEM_FLUID_UOLD][c] + dt * (aRK * RHSu + bRK * F->f[IBMDEM_FLUID_RHSUL][c] - cRK * Px);
        nv[c] = F->f[IBMDEM_FLUID_VOLD][c] + dt * (aRK * RHSv + bRK * F->f[IBMDEM_FLUID_RHSVL][c] - cRK * Py);
        nw[c] = F->f[IBMDEM_FLUID_WOLD][c] + dt * (aRK * RHSw + bRK * F->f[IBMDEM_FLUID_RHSWL][c] - cRK * Pz);
        F->f[IBMDEM_FLUID_PX][c] = Px;
        F->f[IBMDEM_FLUID_PY][c] = Py;
        F->f[IBMDEM_FLUID_PZ][c] = Pz;
        /* RHSul = RHSu after the loop (fluid.F90:130-132): no node reads RHSul
         * of another node, so it is stored here */
        F->f[IBMDEM_FLUID_RHSUL][c] = RHSu;
        F->f[IBMDEM_FLUID_RHSVL][c] = RHSv;
        F->f[IBMDEM_FLUID_RHSWL][c] = RHSw;
      }
  LOOP_INTERIOR {
    const int64_t c = fx_(F, i, j, k);
    U[c] = nu[c];
    V[c] = nv[c];
    W[c] = nw[c];
  }
  free(nu);
}

/* VelocityDivergence (fluid.F90:93-106) */
void orc_fluid_VelocityDivergence(orc_fluid* F, double cRK) {
  const double dx = F->dx, dy = F->dy, dz = F->dz, dt = F->dt, rhof = F->rhof;
  double* dv = F->f[IBMDEM_FLUID_VELDIV];
#pragma omp parallel for schedule(static)
  for (int k = F->SG[2]; k <= F->EG[2]; ++k)
    for (int j = F->SG[1]; j <= F->EG[1]; ++j)
      for (int i = F->SG[0]; i <= F->EG[0]; ++i) {
        const int64_t c = fx_(F, i, j, k);
        double t = (U[fx_(F, i + 1, j, k)] - U[c]) / dx + (V[fx_(F, i, j + 1, k)] - V[c]) / dy +
                   (W[fx_(F, i, j, k + 1)] - W[c]) / dz;
        dv[c] = -t / dt / cRK * rhof;
      }
}

/* ModifyBulkVelocity (fluid.F90:155-195): the interior sums in array order
 * with one accumulator (gfortran's SUM), then a uniform shift of the
 * switched components. */
void orc_fluid_ModifyBulkVelocity(orc_fluid* F, int swU, int swV, int swW, double bulkU, double bulkV,
                                  double bulkW) {
  if (!(swU == 1 || swV == 1 || swW == 1)) return;
  double su = 0.0, sv = 0.0, sw = 0.0;
  LOOP_INTERIOR su = su + U[fx_(F, i, j, k)];
  LOOP_INTERIOR sv = sv + V[fx_(F, i, j, k)];
  LOOP_INTERIOR sw = sw + W[fx_(F, i, j, k)];
  const int nTot = F->n[0] * F->n[1] * F->n[2];
  double mx = 0.0, my = 0.0, mz = 0.0;
  if (swU == 1) mx = -(su / nTot - bulkU) / F->dt;
  if (swV == 1) my = -(sv / nTot - bulkV) / F->dt;
  if (swW == 1) mz = -(sw / nTot - bulkW) / F->dt;
  const double dt = F->dt;
  LOOP_INTERIOR {
    const int64_t c = fx_(F, i, j, k);
    U[c] = U[c] + dt * mx;
    V[c] = V[c] + dt * my;
    W[c] = W[c] + dt * mz;
  }
}

/* PressureCorrection (fluid.F90:197-208) */
void orc_fluid_PressureCorrection(orc_fluid* F) {
  double *P = F->f[IBMDEM_FLUID_P], *Pc = F->f[IBMDEM_FLUID_PCORR];
  LOOP_INTERIOR {
    const int64_t c = fx_(F, i, j, k);
    P[c] = P[c] + Pc[c];
  }
}

/* VelocityCorrection (fluid.F90:210-237): the velocity update, then the
 * vorticity of the corrected field */
void orc_fluid_VelocityCorrection(orc_fluid* F, double cRK) {
  const double dx = F->dx, dy = F->dy, dz = F->dz, dt = F->dt, rhof = F->rhof;
  const double* P = F->f[IBMDEM_FLUID_P];
  const double *Px = F->f[IBMDEM_FLUID_PX], *Py = F->f[IBMDEM_FLUID_PY], *Pz = F->f[IBMDEM_FLUID_PZ];
#pragma omp parallel for schedule(static)
  for (int k = F->SG[2]; k <= F->EG[2]; ++k)
    for (int j = F->SG[1]; j <= F->EG[1]; ++j)
      for (int i = F->SG[0]; i <= F->EG[0]; ++i) {
        const int64_t c = fx_(F, i, j, k);
        U[c] = U[c] + cRK * Px[c] * dt - cRK * (P[c] - P[fx_(F, i - 1, j, k)]) / (dx) * dt / rhof;
        V[c] = V[c] + cRK * Py[c] * dt - cRK * (P[c] - P[fx_(F, i, j - 1, k)]) / (dy) * dt / rhof;
        W[c] = W[c] + cRK * Pz[c] * dt - cRK * (P[c] - P[fx_(F, i, j, k - 1)]) / (dz) * dt / rhof;
      }
  double *ox = F->f[IBMDEM_FLUID_OMEGAX], *oy = F->f[IBMDEM_FLUID_OMEGAY], *oz = F->f[IBMDEM_FLUID_OMEGAZ];
#pragma omp parallel for schedule(static)
  for (int k = F->SG[2]; k <= F->EG[2]; ++k)
    for (int j = F->SG[1]; j <= F->EG[1]; ++j)
      for (int i = F->SG[0]; i <= F->EG[0]; ++i) {
        const int64_t c = fx_(F, i, j, k);
        ox[c] = (W[fx_(F, i, j + 1, k)] - W[c]) / dy - (V[fx_(F, i, j, k + 1)] - V[c]) / dz;
        oy[c] = (U[fx_(F, i, j, k + 1)] - U[c]) / dz - (W[fx_(F, i + 1, j, k)] - W[c]) / dx;
        oz[c] = (V[fx_(F, i + 1, j, k)] - V[c]) / dx - (U[fx_(F, i, j + 1, k)] - U[c]) / dy;
      }
}

/* FillGhostRegionForFluid (boundary.F90:122-147) on one rank: face by face
 * (side 1..6), the halo beyond face sideRecv takes the layers next to face
 * sideSend (periodic, MPISendAndRecvFluidInfo) or, across a wall, the layers
 * next to sideRecv itself mirrored about the face (DealWithBoundaryFluid,
 * boundary.F90:211-245), with u,v,w negated there.  The fields carried are
 * u, v, w, P, omegaZ and Pcorr (errorU/V/P are not used by the stencils).
 * The boxes follow BuildMPIRecvAndSendIndexForFluid (boundary.F90:2-120): the
 * axes of earlier faces with their halo, the later ones interior only. */
static void fbox(const orc_fluid* F, int side, int recv, int wall, int lo[3], int hi[3], int inc[3]) {
  int d = side / 2, high = side % 2;
  for (int e = 0; e < 3; ++e) {
    inc[e] = 1;
    lo[e] = e < d ? F->LG[e] : F->SG[e];
    hi[e] = e < d ? F->UG[e] : F->EG[e];
  }
  if (!recv) {
    lo[d] = high ? F->EG[d] - FHALO + 1 : F->SG[d];
    hi[d] = high ? F->EG[d] : F->SG[d] + FHALO - 1;
  } else if (!wall) {
    lo[d] = high ? F->EG[d] + 1 : F->LG[d];
    hi[d] = high ? F->UG[d] : F->SG[d] - 1;
  } else {
    lo[d] = high ? F->UG[d] : F->SG[d] - 1;
    hi[d] = high ? F->EG[d] + 1 : F->LG[d];
    inc[d] = -1;
  }
}

void orc_fluid_FillGhostRegionForFluid(orc_fluid* F) {
  static const int carried[6] = {IBMDEM_FLUID_U, IBMDEM_FLUID_V, IBMDEM_FLUID_W,
                                 IBMDEM_FLUID_P, IBMDEM_FLUID_OMEGAZ, IBMDEM_FLUID_PCORR};
  for (int s = 0; s < 6; ++s) {
    int sideSend = s, sideRecv = (s % 2 == 0) ? s + 1 : s - 1;
    int wall = F->bType[sideRecv] == 1;
    int from = wall ? sideRecv : sideSend;
    int slo[3], shi[3], sinc[3], rlo[3], rhi[3], rinc[3];
    fbox(F, from, 0, 0, slo, shi, sinc);
    fbox(F, sideRecv, 1, wall, rlo, rhi, rinc);
    int d = sideRecv / 2;
    int nr = (rhi[d] - rlo[d]) * rinc[d] + 1;
    for (int k = slo[2]; k <= shi[2]; ++k)
      for (int j = slo[1]; j <= shi[1]; ++j)
        for (int ii = slo[0]; ii <= shi[0]; ++ii) {
          int src[3] = {ii, j, k}, dst[3] = {ii, j, k};
          int t = src[d] - slo[d];
          if (t >= nr) continue;
          dst[d] = rlo[d] + t * rinc[d];
          int64_t a = fx_(F, dst[0], dst[1], dst[2]), s0 = fx_(F, src[0], src[1], src[2]);
          for (int q = 0; q < 6; ++q) {
            double* f = F->f[carried[q]];
            f[a] = (wall && q < 3) ? -f[s0] : f[s0];
          }
        }
  }
}

/* Boundary (fluid.F90:240-249) */
void orc_fluid_Boundary(orc_fluid* F) {
  for (int side = 0; side < 6; ++side) {
    if (F->bType[side] != 1) continue;
    int d = side / 2;
    double* f = F->f[IBMDEM_FLUID_U + d];
    int lo[3] = {F->LG[0], F->LG[1], F->LG[2]}, hi[3] = {F->UG[0], F->UG[1], F->UG[2]};
    if (side % 2 == 0) hi[d] = F->SG[d];
    else lo[d] = F->EG[d] + 1;
    for (int k = lo[2]; k <= hi[2]; ++k)
      for (int j = lo[1]; j <= hi[1]; ++j)
        for (int i = lo[0]; i <= hi[0]; ++i) f[fx_(F, i, j, k)] = 0.0;
  }
}

/* The matrix of SetPressureCorrectionJacobian (poisson.F90:50-108) applied to
 * p (field layout) into out (interior nodes; the rest left as it is): each
 * row but global cell 0 -- interior node (1,1,1) -- holds -1/dl^2 for each
 * neighbour of GlobalNeighCellIndex (initialization.F90:105-170: periodic
 * wrap, absent behind a face of bType 1) and minus their sum on the
 * diagonal; the row of cell 0 is the identity (pConstIdx = 1).  Used to check
 * a solve against the reference's own linear system. */
void orc_fluid_PressureOperator(orc_fluid* F, const double* p, double* out) {
  const double dl[3] = {F->dx, F->dy, F->dz};
  LOOP_INTERIOR {
    const int64_t c = fx_(F, i, j, k);
    if (i == 1 && j == 1 && k == 1) {
      out[c] = p[c];
      continue;
    }
    double vc = 0.0, acc = 0.0;
    for (int l = 1; l <= 6; ++l) {
      const int dim = (l + 1) / 2;
      const int sh = 2 * ((l + 1) % 2) - 1;
      int ijk[3] = {i, j, k};
      ijk[dim - 1] += sh;
      const int n = F->n[dim - 1];
      if (ijk[dim - 1] < 1 || ijk[dim - 1] > n) {
        if (F->bType[l - 1] == 1) continue;
        ijk[dim - 1] = (ijk[dim - 1] + n - 1) % n + 1;
      }
      const double value = -1.0 / (dl[dim - 1] * dl[dim - 1]);
      acc = acc + value * p[fx_(F, ijk[0], ijk[1], ijk[2])];
      vc = vc + value;
    }
    vc = -vc;
    out[c] = acc + vc * p[c];
  }
}
