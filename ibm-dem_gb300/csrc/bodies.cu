// bodies.cu — per-body force/torque reduction and rigid-body motion.
//
// AssembleLocalForceMS (ZJS_MS_DEM.F90:494-519) sums, per body and in part
// order, fdrag*vol*rhof, fcol, (x-X) x (fdrag*vol) and (x-X) x fcol.  Every
// body's locals are listed in part order (bodyItems, built with the cell
// lists); lanes of a warp form the per-parcel terms in parallel and fold each
// of the 12 sums sequentially in that order, so the sums are bit-identical to
// the reference's serial loop.
// CloudEvolutionMS / EvolutionMS / ResetVelocityAndPositionLagrangianPoints /
// AdjustParcelPosition follow couplesolverCylinder.F90:2-74,189-217 and
// ZJS_EVOLUTION_DEM.F90:121-150 statement by statement.
//
// Body-relative marker vectors use the periodic image of the body centre that
// is nearest to the marker.  For a body that does not straddle a periodic face
// this is the centre itself, as in the reference; for one that does, the
// one-rank reference would use a vector one box length long.
#include "common.cuh"
#include "kernels.cuh"

namespace ibmdem {

namespace {

// Two bodies a warp, one per half.  Each round a half forms the per-parcel
// terms of its body's next 16 parcels (one a lane, every term exactly as in
// the reference) into shared memory, then lane s < NS of the half folds sum s
// over those 16 in part order.  WHICH selects the sums: 1 = fdrag and fmom
// (the hydrodynamic ones), 2 = fcol and fmomCol, 3 = all twelve.  (Four bodies
// a warp, with 8 or 32 parcels a round, measured slower: the fold is a
// dependent chain per sum.)  One warp per block: the body pairs spread over
// all SMs.
constexpr int kSumWarps = 1;
constexpr int kSumBatch = 16;  // parcels per round, one per lane of a half
template <int WHICH>
__global__ void __launch_bounds__(kSumWarps * 32) k_body_sums(Recs R, Geom g, ibmdem_multisphere* B, int nMS,
                                                              const int* __restrict__ bodyStart,
                                                              const int* __restrict__ bodyItems) {
  constexpr int NS = WHICH == 3 ? 12 : 6;  // sums per body
  constexpr int G = kSumBatch;             // lanes per body
  constexpr int SH = 4;                    // log2(G)
  __shared__ double term[kSumWarps][32 / G][kSumBatch][NS + 1];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int grp = lane >> SH, hl = lane & (G - 1);
  const int b = (blockIdx.x * kSumWarps + warp) * (32 / G) + grp;
  const bool hasBody = b < nMS;
  double X[3] = {0.0, 0.0, 0.0};
  int q0 = 0, q1 = 0;
  if (hasBody) {
    for (int k = 0; k < 3; ++k) X[k] = B[b].x[k];
    q0 = bodyStart[b];
    q1 = bodyStart[b + 1];
  }
  const double rhof = g.rhof;
  double acc = 0.0;  // lane hl < NS owns sum hl
  int maxRounds = (q1 - q0 + kSumBatch - 1) / kSumBatch;
#pragma unroll
  for (int o = G; o < 32; o <<= 1) maxRounds = max(maxRounds, __shfl_xor_sync(0xffffffffu, maxRounds, o));
  double(*T)[NS + 1] = term[warp][grp];
  for (int rd = 0; rd < maxRounds; ++rd) {
    const int base = q0 + kSumBatch * rd;
    const int q = base + hl;
    if (q < q1) {
      const int m = bodyItems[q];
      double rpc[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double x = R.D(D_X + k, m);
        rpc[k] = x - body_ref(g, k, x, X[k]);
      }
      double* t = T[hl];
      // terms in output order: WHICH 3 is fdrag, fcol, fmom, fmomCol; WHICH 1
      // fdrag, fmom; WHICH 2 fcol, fmomCol
      if (WHICH & 1) {
        const double vol = R.D(D_VOL, m);
        double fd[3], fv[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          fd[k] = R.D(D_FDRAG + k, m);
          fv[k] = fd[k] * vol;
          t[k] = fd[k] * vol * rhof;
        }
        // CrossMultiplication (ZJS_AUXILIARY_DEM.F90:20-30)
        double* tm = t + (WHICH == 3 ? 6 : 3);
        tm[0] = rpc[1] * fv[2] - rpc[2] * fv[1];
        tm[1] = -rpc[0] * fv[2] + rpc[2] * fv[0];
        tm[2] = rpc[0] * fv[1] - rpc[1] * fv[0];
      }
      if (WHICH & 2) {
        double fc[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) fc[k] = R.D(D_FCOL + k, m);
        double* tc = t + (WHICH == 3 ? 3 : 0);
        double* tcm = t + (WHICH == 3 ? 9 : 3);
#pragma unroll
        for (int k = 0; k < 3; ++k) tc[k] = fc[k];
        tcm[0] = rpc[1] * fc[2] - rpc[2] * fc[1];
        tcm[1] = -rpc[0] * fc[2] + rpc[2] * fc[0];
        tcm[2] = rpc[0] * fc[1] - rpc[1] * fc[0];
      }
    }
    __syncwarp();
    const int n = min(kSumBatch, q1 - base);
    if (hl < NS)
      for (int j = 0; j < n; ++j) acc = acc + T[j][hl];
    __syncwarp();
  }
  if (!hasBody || hl >= NS) return;
  const int which = hl / 3, k = hl - 3 * which;
  double* out;
  if (WHICH == 3)
    out = which == 0 ? B[b].fdrag : which == 1 ? B[b].fcol : which == 2 ? B[b].fmom : B[b].fmomCol;
  else if (WHICH == 1)
    out = which == 0 ? B[b].fdrag : B[b].fmom;
  else
    out = which == 0 ? B[b].fcol : B[b].fmomCol;
  out[k] = acc;
}

// CloudEvolutionMS before AssembleForceMS (couplesolverCylinder.F90:194-204)
__global__ void k_cloud_pre(Geom g, ibmdem_multisphere* B, int nMS) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nMS) return;
  ibmdem_multisphere& M = B[b];
  double ratio = (M.rho - g.rhof) / M.rho;
  for (int k = 0; k < 3; ++k) {
    M.fhydro[k] = (M.v[k] - M.vold[k]) / g.dt * (1.0 - ratio);
    M.fmomHydro[k] = (M.AngMom[k] - M.AngMomOld[k]) / g.dt * (1.0 - ratio);
    M.vold[k] = M.v[k];
    M.AngMomOld[k] = M.AngMom[k];
  }
}

// CloudEvolutionMS after AssembleForceMS (couplesolverCylinder.F90:208-211)
__global__ void k_cloud_post(ibmdem_multisphere* B, int nMS) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nMS) return;
  ibmdem_multisphere& M = B[b];
  for (int k = 0; k < 3; ++k) {
    M.fhydro[k] = M.fhydro[k] + M.fdrag[k] / M.m;
    M.fmomHydro[k] = M.fmomHydro[k] + M.fmom[k];
  }
}

__device__ inline void tensor_mul(const double* A, const double* Bm, double* D) {
  double C[9];
  C[0] = A[0] * Bm[0] + A[1] * Bm[3] + A[2] * Bm[6];
  C[1] = A[0] * Bm[1] + A[1] * Bm[4] + A[2] * Bm[7];
  C[2] = A[0] * Bm[2] + A[1] * Bm[5] + A[2] * Bm[8];
  C[3] = A[3] * Bm[0] + A[4] * Bm[3] + A[5] * Bm[6];
  C[4] = A[3] * Bm[1] + A[4] * Bm[4] + A[5] * Bm[7];
  C[5] = A[3] * Bm[2] + A[4] * Bm[5] + A[5] * Bm[8];
  C[6] = A[6] * Bm[0] + A[7] * Bm[3] + A[8] * Bm[6];
  C[7] = A[6] * Bm[1] + A[7] * Bm[4] + A[8] * Bm[7];
  C[8] = A[6] * Bm[2] + A[7] * Bm[5] + A[8] * Bm[8];
  for (int q = 0; q < 9; ++q) D[q] = C[q];
}

// EvolutionMS (couplesolverCylinder.F90:2-42) with CalculateRotateMatrix (:76-97)
__global__ void k_evolution(Geom g, ibmdem_multisphere* B, int nMS) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= nMS) return;
  ibmdem_multisphere& M = B[b];
  const double dtDEM = g.dtDEM;
  double ratio = (M.rho - g.rhof) / M.rho;
  for (int q = 0; q < 9; ++q) M.rotMatGloOld[q] = M.rotMatGlo[q];
  for (int k = 0; k < 3; ++k)
    M.v[k] = M.v[k] + M.fhydro[k] * dtDEM + M.fcol[k] / M.m * dtDEM + ratio * g.g[k] * dtDEM;
  {
    double th0 = M.omega[0] * dtDEM, th1 = M.omega[1] * dtDEM, th2 = M.omega[2] * dtDEM;
    double mag = sqrt(th0 * th0 + th1 * th1 + th2 * th2);
    mag = fmax(mag, 1e-10);
    double ux = th0 / mag, uy = th1 / mag, uz = th2 / mag;
    double cm = cos(mag), sm = sin(mag);
    double* mat = M.rotMat;
    mat[0] = (1 - cm) * ux * ux + cm;
    mat[1] = (1 - cm) * ux * uy - sm * uz;
    mat[2] = (1 - cm) * ux * uz + sm * uy;
    mat[3] = (1 - cm) * uy * ux + sm * uz;
    mat[4] = (1 - cm) * uy * uy + cm;
    mat[5] = (1 - cm) * uy * uz - sm * ux;
    mat[6] = (1 - cm) * uz * ux - sm * uy;
    mat[7] = (1 - cm) * uz * uy + sm * ux;
    mat[8] = (1 - cm) * uz * uz + cm;
  }
  double ITInv[9], RMInv[9], TMInvTmp[9], TMInv[9];
  for (int q = 0; q < 9; ++q) ITInv[q] = M.InertiaTensor[q];
  ITInv[0] = 1.0 / ITInv[0];
  ITInv[4] = 1.0 / ITInv[4];
  ITInv[8] = 1.0 / ITInv[8];
  tensor_mul(M.rotMatGlo, M.rotMat, M.rotMatGlo);
  const double* A = M.rotMatGlo;
  RMInv[0] = A[0]; RMInv[1] = A[3]; RMInv[2] = A[6];
  RMInv[3] = A[1]; RMInv[4] = A[4]; RMInv[5] = A[7];
  RMInv[6] = A[2]; RMInv[7] = A[5]; RMInv[8] = A[8];
  tensor_mul(M.rotMatGlo, ITInv, TMInvTmp);
  tensor_mul(TMInvTmp, RMInv, TMInv);
  for (int k = 0; k < 3; ++k) M.AngMom[k] = M.AngMom[k] + (M.fmomHydro[k] + M.fmomCol[k]) * dtDEM;
  double c1 = TMInv[0] * M.AngMom[0] + TMInv[1] * M.AngMom[1] + TMInv[2] * M.AngMom[2];
  double c2 = TMInv[3] * M.AngMom[0] + TMInv[4] * M.AngMom[1] + TMInv[5] * M.AngMom[2];
  double c3 = TMInv[6] * M.AngMom[0] + TMInv[7] * M.AngMom[1] + TMInv[8] * M.AngMom[2];
  M.omega[0] = c1;
  M.omega[1] = c2;
  M.omega[2] = c3;
  for (int k = 0; k < 3; ++k) M.x[k] = M.x[k] + M.v[k] * dtDEM;
}

// ResetVelocityAndPositionLagrangianPoints (couplesolverCylinder.F90:44-74)
// and/or AdjustParcelPosition (ZJS_EVOLUTION_DEM.F90:121-150)
__global__ void k_marker_update(Recs R, Geom g, const Counters* cnt, const ibmdem_multisphere* B, int reset,
                                int adjust) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= cnt->npLocal) return;
  double x[3] = {R.D(D_X, m), R.D(D_X + 1, m), R.D(D_X + 2, m)};
  if (reset) {
    const ibmdem_multisphere& M = B[R.I(I_MSIDX, m) - 1];
    const double dtDEM = g.dtDEM;
    for (int k = 0; k < 3; ++k) x[k] = x[k] + M.v[k] * dtDEM;
    double xc[3], xt[3];
    for (int k = 0; k < 3; ++k) xc[k] = body_ref(g, k, x[k], M.x[k]);
    for (int k = 0; k < 3; ++k) xt[k] = x[k] - xc[k];
    const double* mat = M.rotMat;
    x[0] = mat[0] * xt[0] + mat[1] * xt[1] + mat[2] * xt[2];
    x[1] = mat[3] * xt[0] + mat[4] * xt[1] + mat[5] * xt[2];
    x[2] = mat[6] * xt[0] + mat[7] * xt[1] + mat[8] * xt[2];
    for (int k = 0; k < 3; ++k) x[k] = x[k] + xc[k];
    double r[3] = {x[0] - xc[0], x[1] - xc[1], x[2] - xc[2]};
    const double* a = M.omega;
    double c1 = a[1] * r[2] - a[2] * r[1];
    double c2 = -a[0] * r[2] + a[2] * r[0];
    double c3 = a[0] * r[1] - a[1] * r[0];
    R.D(D_V, m) = c1 + M.v[0];
    R.D(D_V + 1, m) = c2 + M.v[1];
    R.D(D_V + 2, m) = c3 + M.v[2];
  }
  if (adjust) {
    for (int d = 0; d < 3; ++d) {
      if (fabs(x[d] - g.start[d]) < g.err[d]) x[d] = g.start[d] + g.err[d];
      if (fabs(x[d] - g.end[d]) < g.err[d]) x[d] = g.end[d] + g.err[d];
    }
  }
  for (int k = 0; k < 3; ++k) R.D(D_X + k, m) = x[k];
}

}  // namespace

void launch_body_sums(Ctx& c, int which) {
  if (c.nMS <= 0) return;
  const int perWarp = 2;
  auto k = which == SUMS_ALL ? k_body_sums<3> : which == SUMS_HYDRO ? k_body_sums<1> : k_body_sums<2>;
  k<<<nblocks((c.nMS + perWarp - 1) / perWarp, kSumWarps), kSumWarps * 32, 0, c.stream>>>(c.rec(), c.g, c.dBodies,
                                                                                         c.nMS, c.bodyStart,
                                                                                         c.bodyItems);
  c.launches++;
}

void launch_evolution(Ctx& c) {
  if (c.nMS <= 0) return;
  k_evolution<<<nblocks(c.nMS, 64), 64, 0, c.stream>>>(c.g, c.dBodies, c.nMS);
  c.launches++;
}

void launch_cloud_pre(Ctx& c) {
  if (c.nMS <= 0) return;
  k_cloud_pre<<<nblocks(c.nMS, 64), 64, 0, c.stream>>>(c.g, c.dBodies, c.nMS);
  c.launches++;
}

void launch_cloud_post(Ctx& c) {
  if (c.nMS <= 0) return;
  k_cloud_post<<<nblocks(c.nMS, 64), 64, 0, c.stream>>>(c.dBodies, c.nMS);
  c.launches++;
}

void launch_marker_update(Ctx& c, bool reset, bool adjust) {
  k_marker_update<<<nblocks(c.capLocal), kBlock, 0, c.stream>>>(c.rec(), c.g, c.dCnt, c.dBodies, reset ? 1 : 0,
                                                                adjust ? 1 : 0);
  c.launches++;
}

}  // namespace ibmdem
