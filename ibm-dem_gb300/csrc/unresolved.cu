// unresolved.cu — the unresolved CFD-DEM path: point particles with
// spring-dashpot contacts, Coulomb friction and tangential history, a
// Gaussian-kernel solid volume fraction on the fluid cells, and the drag law of
// CalculateDragForce (ZJS_DRAGFORCE_DEM.F90:2-35) against a frozen fluid.
//
// Data layout: particle state is field-major (one array per scalar field,
// np long); contact history is particle-major with maxContacts slots per
// particle, double-buffered between steps.  Two cell lists per step, the DEM
// cells (contacts) and the fluid cells (volume fraction), each in part order
// within a cell (slots from the count atomics, a scatter and a per-cell order
// fix-up: the order a stable sort gives); both gathers then walk particles in
// part order within a cell.
//
// Every sum has a fixed order, so results do not depend on scheduling:
//   fcol, tcol  over the 27 neighbour DEM cells (z outermost, periodic) and,
//               within a cell, part order;
//   alphap      per source fluid cell over its particles in part order (the
//               cell stamp), then over the 125 source cells at offsets
//               (dz,dy,dx) in -2..2 (z outermost).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "common.cuh"
#include "prims.cuh"

namespace ibmdem {
namespace {

// particle fields (field-major, np doubles each)
enum UField : int {
  U_RAD = 0, U_RHO, U_VOL, U_M, U_I, U_X, U_V = U_X + 3, U_W = U_V + 3, U_FCOL = U_W + 3, U_TCOL = U_FCOL + 3,
  U_FDRAG = U_TCOL + 3, U_ALPHA = U_FDRAG + 3, U_ND
};

constexpr int UE_RANGE = 1;     // a particle outside the periodic box (or NaN)
constexpr int UE_CONTACTS = 2;  // more touching partners than maxContacts

struct UGeom {
  int n[3];            // fluid cells
  int ni, nj;          // fluid array extents with the 2-cell halo (x, y)
  long long nint;      // fluid interior cells
  double h, vcell;     // fluid cell size and volume
  double L[3], halfL[3];
  int nc[3];           // DEM cells per axis
  double cs[3];        // DEM cell size per axis
  long long ncd;       // DEM cells
  int K;               // history slots per particle
  double dt, rhof, viscf, knCoeff, knScale, eta, ktRatio, mu, bandwidth, alphaMin, grav[3];
};

struct UPtr {
  double* d;  // [U_ND * cap]
  int* gidx;
  int cap;
  __device__ double& D(int f, int i) const { return d[(size_t)f * cap + i]; }
};

__device__ inline void uset_err(int* err, int bit, int* info, int i) {
  if (atomicOr(err, bit) == 0) *info = i;
}

__device__ inline int dem_cell_axis(const UGeom& g, int d, double x) {
  int c = (int)floor(x / g.cs[d]);
  return min(max(c, 0), g.nc[d] - 1);
}

__device__ inline double min_image(double d, double L, double halfL) {
  if (d > halfL) return d - L;
  if (d < -halfL) return d + L;
  return d;
}

// Cell keys for both cell lists, and each particle's slot in its cells from
// the count atomics; positions outside [0, L) are flagged.  The lists are
// built without a sort: the scans of the counts give the cells' starts, every
// particle goes to start + slot, and the particle that took slot 0 puts its
// cell's few items back in index order -- the order a stable sort by cell
// gives.
__global__ void k_u_keys(UGeom g, UPtr P, int np, uint32_t* kd, uint32_t* vd, int* cntD, uint32_t* kf,
                         uint32_t* vf, int* cntF, int* err, int* info) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  int cd[3], cf[3];
  bool ok = true;
  for (int d = 0; d < 3; ++d) {
    double x = P.D(U_X + d, i);
    ok = ok && x >= 0.0 && x < g.L[d];
    cd[d] = ok ? dem_cell_axis(g, d, x) : 0;
    int f = ok ? (int)floor(x / g.h) : 0;
    cf[d] = min(max(f, 0), g.n[d] - 1);
  }
  if (!ok) uset_err(err, UE_RANGE, info, i);
  uint32_t keyD = (uint32_t)(((long long)cd[2] * g.nc[1] + cd[1]) * g.nc[0] + cd[0]);
  uint32_t keyF = (uint32_t)(((long long)cf[2] * g.n[1] + cf[1]) * g.n[0] + cf[0]);
  kd[i] = keyD;
  kf[i] = keyF;
  vd[i] = (uint32_t)atomicAdd(&cntD[keyD], 1);
  vf[i] = (uint32_t)atomicAdd(&cntF[keyF], 1);
}

// particle i to its cell's start + slot; the cell's count goes back to zero
// for the next step
__global__ void k_u_place(int np, const uint32_t* __restrict__ key, const uint32_t* __restrict__ slot,
                          const int* __restrict__ start, int* items, int* count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  items[start[key[i]] + (int)slot[i]] = i;
  if (slot[i] == 0) count[key[i]] = 0;
}

// the slot-0 particle of each cell sorts the cell's items by index (Shell sort
// with Ciura's gaps: an insertion sort for the usual handful)
__global__ void k_u_order(int np, const uint32_t* __restrict__ key, const uint32_t* __restrict__ slot,
                          const int* __restrict__ start, int* items) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np || slot[i] != 0) return;
  const uint32_t c = key[i];
  const int s0 = start[c], n = start[c + 1] - s0;
  if (n < 2) return;
  int* a = items + s0;
  constexpr int kGaps[8] = {701, 301, 132, 57, 23, 10, 4, 1};
  for (int gi = 0; gi < 8; ++gi) {
    const int gap = kGaps[gi];
    for (int q = gap; q < n; ++q) {
      const int v = a[q];
      int j = q;
      while (j >= gap && a[j - gap] > v) {
        a[j] = a[j - gap];
        j -= gap;
      }
      a[j] = v;
    }
  }
}

// Positions and radii in DEM-cell order, rounded to FP32, for the search.
__global__ void k_u_pos32(UPtr P, int np, const int* __restrict__ items, float4* pos) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= np) return;
  const int i = items[t];
  pos[t] = make_float4((float)P.D(U_X, i), (float)P.D(U_X + 1, i), (float)P.D(U_X + 2, i), (float)P.D(U_RAD, i));
}

// Touching partners of particle i in scan order: 27 neighbour DEM cells (z
// outermost, periodic), part order within a cell.  An FP32 test with a 1e-3
// relative margin keeps the candidates (the FP32 distance differs from the FP64
// one by far less than the margin); after the scan the FP64 test
// d2 < (r_i + r_j)^2 decides each candidate in scan order, so FP64 instructions
// are not issued inside the divergent cell loop.  A particle with more than
// kCand candidates rescans with the FP64 test inline.
constexpr int kCand = 16;
__device__ inline bool touches(const UGeom& g, const UPtr& P, int i, int j) {
  const double r1 = min_image(P.D(U_X, i) - P.D(U_X, j), g.L[0], g.halfL[0]);
  const double r2 = min_image(P.D(U_X + 1, i) - P.D(U_X + 1, j), g.L[1], g.halfL[1]);
  const double r3 = min_image(P.D(U_X + 2, i) - P.D(U_X + 2, j), g.L[2], g.halfL[2]);
  const double rij = P.D(U_RAD, i) + P.D(U_RAD, j);
  return r1 * r1 + r2 * r2 + r3 * r3 < rij * rij;
}

__global__ void __launch_bounds__(kBlock) k_u_find(UGeom g, UPtr P, int np, const int* __restrict__ cellStart,
                                                   const int* __restrict__ items, const float4* __restrict__ pos,
                                                   int* nc, int* partner, int* err, int* info) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= np) return;
  const int i = items[t];
  const float4 pi = pos[t];
  const float Lx = (float)g.L[0], Ly = (float)g.L[1], Lz = (float)g.L[2];
  const float Hx = (float)g.halfL[0], Hy = (float)g.halfL[1], Hz = (float)g.halfL[2];
  // the particle's DEM cell from its FP64 position (as the cell keys)
  const int c0 = dem_cell_axis(g, 0, P.D(U_X, i)), c1 = dem_cell_axis(g, 1, P.D(U_X + 1, i)),
            c2 = dem_cell_axis(g, 2, P.D(U_X + 2, i));
  int cand[kCand];
  int ncand = 0;
  for (int pass = 0; pass < 2; ++pass) {
    int m = 0;
    for (int dz = -1; dz <= 1; ++dz) {
      const int cz = (c2 + dz + g.nc[2]) % g.nc[2];
      for (int dy = -1; dy <= 1; ++dy) {
        const int cy = (c1 + dy + g.nc[1]) % g.nc[1];
        for (int dx = -1; dx <= 1; ++dx) {
          const int cx = (c0 + dx + g.nc[0]) % g.nc[0];
          const long long cell = ((long long)cz * g.nc[1] + cy) * g.nc[0] + cx;
          const int q1 = cellStart[cell + 1];
          for (int q = cellStart[cell]; q < q1; ++q) {
            if (q == t) continue;
            const float4 pj = pos[q];
            float ex = pi.x - pj.x, ey = pi.y - pj.y, ez = pi.z - pj.z;
            ex = ex > Hx ? ex - Lx : (ex < -Hx ? ex + Lx : ex);
            ey = ey > Hy ? ey - Ly : (ey < -Hy ? ey + Ly : ey);
            ez = ez > Hz ? ez - Lz : (ez < -Hz ? ez + Lz : ez);
            const float rf = (pi.w + pj.w) * 1.001f;
            if (ex * ex + ey * ey + ez * ez > rf * rf) continue;
            if (pass == 0) {
              if (ncand < kCand) cand[ncand] = q;
              ++ncand;
            } else {
              const int j = items[q];
              if (!touches(g, P, i, j)) continue;
              if (m < g.K)
                partner[(size_t)i * g.K + m] = j;
              else
                uset_err(err, UE_CONTACTS, info, i);
              ++m;
            }
          }
        }
      }
    }
    if (pass == 1) {
      nc[i] = min(m, g.K);
      return;
    }
    if (ncand <= kCand) break;
  }
  int m = 0;
  for (int c = 0; c < ncand; ++c) {
    const int j = items[cand[c]];
    if (!touches(g, P, i, j)) continue;
    if (m < g.K)
      partner[(size_t)i * g.K + m] = j;
    else
      uset_err(err, UE_CONTACTS, info, i);
    ++m;
  }
  nc[i] = min(m, g.K);
}

// Flat contact list: slot ids (i*K + m) of all touching pairs, particle-major.
__global__ void k_u_owner(int np, int K, const int* __restrict__ nc, const int* __restrict__ cstart, int* owner) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const int n = nc[i], e0 = cstart[i];
  for (int m = 0; m < n; ++m) owner[e0 + m] = i * K + m;
}

// One thread per touching pair (all lanes busy whatever the contact counts):
// the pair's force term fn*n + ft and torque term ri*(n x ft) for particle i,
// and its new tangential displacement.  The tangential displacement continues
// from i's previous slot for the same partner, else starts at zero.
__global__ void __launch_bounds__(kBlock) k_u_pair(UGeom g, UPtr P, const int* __restrict__ total,
                                                   const int* __restrict__ owner, const int* __restrict__ ncOld,
                                                   const int* __restrict__ pOld, const double* __restrict__ xOld,
                                                   const int* __restrict__ pNew, double* xNew, double* fterm,
                                                   double* tterm) {
  const long long nPairs = *total;
  GRID_STRIDE(e, nPairs) {
    const int slot = owner[e];
    const int i = slot / g.K;
    const int j = pNew[slot];
    const double ri = P.D(U_RAD, i), rj = P.D(U_RAD, j);
    const double r1 = min_image(P.D(U_X, i) - P.D(U_X, j), g.L[0], g.halfL[0]);
    const double r2 = min_image(P.D(U_X + 1, i) - P.D(U_X + 1, j), g.L[1], g.halfL[1]);
    const double r3 = min_image(P.D(U_X + 2, i) - P.D(U_X + 2, j), g.L[2], g.halfL[2]);
    const double rij = ri + rj;
    const double d2 = r1 * r1 + r2 * r2 + r3 * r3;
    const double dist = sqrt(d2);
    const double n1 = r1 / dist, n2 = r2 / dist, n3 = r3 / dist;
    const double mi = P.D(U_M, i), mj = P.D(U_M, j);
    const double meff = 2 * mi * mj / (mi + mj);
    const double deltan = rij - dist;
    const double kn = g.knScale * meff;  // knCoeff/(0.1*dx)*meff
    const double etan = g.eta * sqrt(meff * kn);
    const double u1 = P.D(U_V, i) - P.D(U_V, j), u2 = P.D(U_V + 1, i) - P.D(U_V + 1, j),
                 u3 = P.D(U_V + 2, i) - P.D(U_V + 2, j);
    const double vn = n1 * u1 + n2 * u2 + n3 * u3;
    const double fn = kn * deltan - etan * vn;
    // relative velocity of the contact point: u - (ri wi + rj wj) x n
    const double s1 = ri * P.D(U_W, i) + rj * P.D(U_W, j);
    const double s2 = ri * P.D(U_W + 1, i) + rj * P.D(U_W + 1, j);
    const double s3 = ri * P.D(U_W + 2, i) + rj * P.D(U_W + 2, j);
    const double vr1 = u1 - (s2 * n3 - s3 * n2);
    const double vr2 = u2 - (s3 * n1 - s1 * n3);
    const double vr3 = u3 - (s1 * n2 - s2 * n1);
    const double vrn = n1 * vr1 + n2 * vr2 + n3 * vr3;
    const double vt1 = vr1 - vrn * n1, vt2 = vr2 - vrn * n2, vt3 = vr3 - vrn * n3;
    double h1 = 0, h2 = 0, h3 = 0;
    const int nOld = ncOld[i];
    for (int s = 0; s < nOld; ++s)
      if (pOld[(size_t)i * g.K + s] == j) {
        const double* o = xOld + ((size_t)i * g.K + s) * 3;
        h1 = o[0];
        h2 = o[1];
        h3 = o[2];
        break;
      }
    const double hn = n1 * h1 + n2 * h2 + n3 * h3;
    h1 = h1 - hn * n1;
    h2 = h2 - hn * n2;
    h3 = h3 - hn * n3;
    h1 = h1 + g.dt * vt1;
    h2 = h2 + g.dt * vt2;
    h3 = h3 + g.dt * vt3;
    const double kt = g.ktRatio * kn;
    const double etat = g.eta * sqrt(meff * kt);
    double ft1 = -kt * h1 - etat * vt1, ft2 = -kt * h2 - etat * vt2, ft3 = -kt * h3 - etat * vt3;
    const double ftm = sqrt(ft1 * ft1 + ft2 * ft2 + ft3 * ft3);
    const double lim = g.mu * fabs(fn);
    if (ftm > lim) {
      const double sc = lim / ftm;
      ft1 = ft1 * sc;
      ft2 = ft2 * sc;
      ft3 = ft3 * sc;
      h1 = -(ft1 + etat * vt1) / kt;
      h2 = -(ft2 + etat * vt2) / kt;
      h3 = -(ft3 + etat * vt3) / kt;
    }
    double* xo = xNew + (size_t)slot * 3;
    xo[0] = h1;
    xo[1] = h2;
    xo[2] = h3;
    double* fo = fterm + (size_t)slot * 3;
    fo[0] = fn * n1 + ft1;
    fo[1] = fn * n2 + ft2;
    fo[2] = fn * n3 + ft3;
    double* to = tterm + (size_t)slot * 3;
    to[0] = ri * (n2 * ft3 - n3 * ft2);
    to[1] = ri * (n3 * ft1 - n1 * ft3);
    to[2] = ri * (n1 * ft2 - n2 * ft1);
  }
}

// fcol and tcol of particle i: its pair terms folded in list order
__global__ void k_u_sum(UPtr P, int np, int K, const int* __restrict__ nc, const double* __restrict__ fterm,
                        const double* __restrict__ tterm) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  double f0 = 0, f1 = 0, f2 = 0, t0 = 0, t1 = 0, t2 = 0;
  const int n = nc[i];
  for (int m = 0; m < n; ++m) {
    const double* fo = fterm + ((size_t)i * K + m) * 3;
    const double* to = tterm + ((size_t)i * K + m) * 3;
    f0 = f0 + fo[0];
    f1 = f1 + fo[1];
    f2 = f2 + fo[2];
    t0 = t0 - to[0];
    t1 = t1 - to[1];
    t2 = t2 - to[2];
  }
  P.D(U_FCOL, i) = f0;
  P.D(U_FCOL + 1, i) = f1;
  P.D(U_FCOL + 2, i) = f2;
  P.D(U_TCOL, i) = t0;
  P.D(U_TCOL + 1, i) = t1;
  P.D(U_TCOL + 2, i) = t2;
}

// Per particle, in fluid-cell order (slot t holds particle items[t]): the 1-D
// Gaussian weights gx, gy, gz on the 5 fluid cells around its cell per axis,
// the scale s = vol / (sum of the 125 weights * cell volume), and the partial
// products (s*gz[qz])*gy[qy] that every term ((s*gz)*gy)*gx shares.
// With u_q = (x - xc_q)/sigma and d = h/sigma, u_{q+1} = u_q - d, so
// exp(-u_{q+1}^2/2) = exp(-u_q^2/2) * exp(d u_q) * exp(-d^2/2) and
// exp(d u_{q+1}) = exp(d u_q) * exp(-d^2): three exponentials per axis and one
// per particle give the 15 weights (relative difference from 15 direct
// exponentials of order 1e-15).
constexpr int kStamp = 32;  // 25 partial products, 5 gx, 2 spare
__global__ void k_u_gauss(UGeom g, UPtr P, int np, const int* __restrict__ items, double* st) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= np) return;
  const int i = items[t];
  const double sigma = g.bandwidth * (2.0 * P.D(U_RAD, i));
  const double dd = g.h / sigma;
  const double c2 = exp(-(dd * dd));      // ratio of successive growth factors
  double w[3][5], sum[3];
  for (int d = 0; d < 3; ++d) {
    const double x = P.D(U_X + d, i);
    const int a = min(max((int)floor(x / g.h), 0), g.n[d] - 1);
    const double u0 = (x - ((double)(a - 2) + 0.5) * g.h) / sigma;
    double wq = exp(-0.5 * (u0 * u0));
    double r = exp(dd * u0 - 0.5 * (dd * dd));  // w_{q+1} / w_q at q = 0
    double s = 0.0;
    for (int q = 0; q < 5; ++q) {
      w[d][q] = wq;
      s = s + wq;
      wq = wq * r;
      r = r * c2;
    }
    sum[d] = s;
  }
  const double sc = P.D(U_VOL, i) / (((sum[0] * sum[1]) * sum[2]) * g.vcell);
  double* o = st + (size_t)t * kStamp;
  for (int qz = 0; qz < 5; ++qz)
    for (int qy = 0; qy < 5; ++qy) o[qz * 5 + qy] = (sc * w[2][qz]) * w[1][qy];
  for (int qx = 0; qx < 5; ++qx) o[25 + qx] = w[0][qx];
}

// Occupied fluid cells: flag, then (after an exclusive scan into rank) the list.
__global__ void k_u_occ_flag(long long nint, const int* __restrict__ flStart, int* flag) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < nint) flag[c] = flStart[c + 1] > flStart[c] ? 1 : 0;
}
__global__ void k_u_occ_list(long long nint, const int* __restrict__ flStart, const int* __restrict__ rank,
                             int* occ) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < nint && flStart[c + 1] > flStart[c]) occ[rank[c]] = (int)c;
}

// Cell stamps: for every occupied fluid cell (one warp each) and every offset
// (qz,qy,qx) of the 5x5x5 cells it reaches, the sum over its particles in part
// order of ((s*gz[qz])*gy[qy])*gx[qx].  Lane l holds offsets l, l+32, l+64, l+96.
constexpr int kCellStamp = 128;  // 125 offsets, padded
__global__ void __launch_bounds__(kBlock) k_u_cellsum(const int* __restrict__ nOcc, const int* __restrict__ occ,
                                                      const int* __restrict__ flStart,
                                                      const double* __restrict__ st, double* T) {
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  const int n = *nOcc;
  int pq[4], qx[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int o = min(lane + 32 * r, 124);
    pq[r] = o / 5;       // qz*5 + qy
    qx[r] = o % 5;
  }
  for (long long w = warp; w < n; w += nwarps) {
    const int c = occ[w];
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const int q1 = flStart[c + 1];
    for (int q = flStart[c]; q < q1; ++q) {
      const double* x = st + (size_t)q * kStamp;
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[r] = acc[r] + x[pq[r]] * x[25 + qx[r]];
    }
    double* out = T + (size_t)w * kCellStamp;
#pragma unroll
    for (int r = 0; r < 4; ++r)
      if (lane + 32 * r < 125) out[lane + 32 * r] = acc[r];
  }
}

// alphaf of every fluid cell: alphap = sum over the source cells at offsets
// (dz,dy,dx) in -2..2, z outermost, of their cell stamp at the offset that
// reaches this cell; alphaf = max(1 - alphap, alphaMin).
__global__ void __launch_bounds__(kBlock) k_u_alpha(UGeom g, const int* __restrict__ flStart,
                                                    const int* __restrict__ rank, const double* __restrict__ T,
                                                    double* alphaf) {
  long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.nint) return;
  const int i = (int)(c % g.n[0]);
  const int j = (int)((c / g.n[0]) % g.n[1]);
  const int k = (int)(c / ((long long)g.n[0] * g.n[1]));
  double ap = 0.0;
  for (int oz = -2; oz <= 2; ++oz) {
    const int sz = (k + oz + g.n[2]) % g.n[2];
    for (int oy = -2; oy <= 2; ++oy) {
      const int sy = (j + oy + g.n[1]) % g.n[1];
      const long long row = ((long long)sz * g.n[1] + sy) * g.n[0];
      const int pq5 = ((2 - oz) * 5 + (2 - oy)) * 5;
      for (int ox = -2; ox <= 2; ++ox) {
        const long long src = row + (i + ox + g.n[0]) % g.n[0];
        if (flStart[src + 1] > flStart[src]) ap = ap + T[(size_t)rank[src] * kCellStamp + pq5 + (2 - ox)];
      }
    }
  }
  alphaf[c] = fmax(1.0 - ap, g.alphaMin);
}

// CalculateDragForce (ZJS_DRAGFORCE_DEM.F90:2-35): the literals 3.7, 0.65,
// 0.687, 0.0183, 8.33, 0.0972 and 0.8 are default-real (single precision) there.
// log10(Rep) and Rep**0.687 share log(Rep); alphaf**(-zeta) is
// exp(-zeta*log(alphaf)) with log(alphaf) shared by the three components
// (relative difference from pow/log10 of order 1e-15).
__device__ inline void drag_beta(double rho, double rad, const double* v, double denf, double alphaf, const double* velf,
                                 double viscf, double* beta) {
  const double c37 = (double)3.7f, c065 = (double)0.65f, c0687 = (double)0.687f, c00183 = (double)0.0183f;
  const double c833 = (double)8.33f, c00972 = (double)0.0972f, c08 = (double)0.8f;
  const double inv_ln10 = 0.43429448190325182765;  // 1/ln(10)
  const double spg = rho / denf;
  const double diameter = 2.0 * rad;
  const double la = alphaf < c08 ? 0.0 : log(alphaf);
  for (int j = 0; j < 3; ++j) {
    const double Ur = fabs(velf[j] - v[j]);
    double Rep = Ur * diameter / viscf;
    Rep = Rep > 1.0 ? Rep : 1.0;
    const double lr = log(Rep);
    const double t = 1.5 - lr * inv_ln10;
    const double zeta = c37 - c065 * exp(-0.5 * (t * t));
    double fbase, f;
    if (Rep < 1000)
      fbase = 1 + 1.0 / 6.0 * exp(c0687 * lr);
    else
      fbase = c00183 * Rep;
    if (alphaf < c08)
      f = c833 * (1 - alphaf) / alphaf + c00972 * Rep;
    else
      f = fbase * exp(-zeta * la);
    const double Cd = 24.0 / Rep * f;
    beta[j] = 0.75 * (Cd * Ur) / (diameter * spg);
  }
}

__global__ void k_drag_beta(int n, const double* rho, const double* rad, const double* v, double denf,
                            const double* alphaf, const double* velf, double* beta) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  drag_beta(rho[i], rad[i], v + 3 * (size_t)i, denf, alphaf[i], velf + 3 * (size_t)i, 1e-5, beta + 3 * (size_t)i);
}

__device__ inline double lerp3(const double* F, int ni, int nj, int i0, int j0, int k0, double tx, double ty,
                               double tz) {
  // F at Fortran-with-halo index (i,j,k): ((k+1)*nj + (j+1))*ni + (i+1)
  auto at = [&](int i, int j, int k) { return F[((long long)(k + 1) * nj + (j + 1)) * ni + (i + 1)]; };
  const double sx = 1.0 - tx, sy = 1.0 - ty, sz = 1.0 - tz;
  const double c00 = at(i0, j0, k0) * sx + at(i0 + 1, j0, k0) * tx;
  const double c10 = at(i0, j0 + 1, k0) * sx + at(i0 + 1, j0 + 1, k0) * tx;
  const double c01 = at(i0, j0, k0 + 1) * sx + at(i0 + 1, j0, k0 + 1) * tx;
  const double c11 = at(i0, j0 + 1, k0 + 1) * sx + at(i0 + 1, j0 + 1, k0 + 1) * tx;
  const double c0 = c00 * sy + c10 * ty;
  const double c1 = c01 * sy + c11 * ty;
  return c0 * sz + c1 * tz;
}

// fluid velocity and fraction at the particle, drag, and the time step
__global__ void k_u_drag_move(UGeom g, UPtr P, int np, const double* __restrict__ uf, const double* __restrict__ vf,
                              const double* __restrict__ wf, const double* __restrict__ alphaf) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  double x[3], v[3], vel[3];
  for (int d = 0; d < 3; ++d) {
    x[d] = P.D(U_X + d, i);
    v[d] = P.D(U_V + d, i);
  }
  // MAC faces: component c at (i-1)h along axis c and (i-1/2)h across (Fortran
  // indices, 1-based interior, 2-cell halo)
  const double* F[3] = {uf, vf, wf};
  for (int c = 0; c < 3; ++c) {
    int i0[3];
    double t[3];
    for (int d = 0; d < 3; ++d) {
      const double f = x[d] / g.h + (d == c ? 1.0 : 0.5);
      i0[d] = (int)floor(f);
      t[d] = f - (double)i0[d];
    }
    vel[c] = lerp3(F[c], g.ni, g.nj, i0[0], i0[1], i0[2], t[0], t[1], t[2]);
  }
  // fluid fraction on the cell centres (i+1/2)h, i = 0..n-1, periodic
  int a0[3];
  double ta[3];
  for (int d = 0; d < 3; ++d) {
    const double f = x[d] / g.h - 0.5;
    a0[d] = (int)floor(f);
    ta[d] = f - (double)a0[d];
  }
  auto A = [&](int di, int dj, int dk) {
    const int ii = (a0[0] + di + g.n[0]) % g.n[0];
    const int jj = (a0[1] + dj + g.n[1]) % g.n[1];
    const int kk = (a0[2] + dk + g.n[2]) % g.n[2];
    return alphaf[((long long)kk * g.n[1] + jj) * g.n[0] + ii];
  };
  const double sx = 1.0 - ta[0], sy = 1.0 - ta[1], sz = 1.0 - ta[2];
  const double c00 = A(0, 0, 0) * sx + A(1, 0, 0) * ta[0];
  const double c10 = A(0, 1, 0) * sx + A(1, 1, 0) * ta[0];
  const double c01 = A(0, 0, 1) * sx + A(1, 0, 1) * ta[0];
  const double c11 = A(0, 1, 1) * sx + A(1, 1, 1) * ta[0];
  const double af = (c00 * sy + c10 * ta[1]) * sz + (c01 * sy + c11 * ta[1]) * ta[2];
  double beta[3];
  const double m = P.D(U_M, i), rho = P.D(U_RHO, i), I = P.D(U_I, i);
  drag_beta(rho, P.D(U_RAD, i), v, g.rhof, af, vel, g.viscf, beta);
  const double ratio = 1.0 - g.rhof / rho;
  for (int d = 0; d < 3; ++d) {
    const double fd = (m * beta[d]) * (vel[d] - v[d]);
    P.D(U_FDRAG + d, i) = fd;
    double a = (fd + P.D(U_FCOL + d, i)) / m;
    a = a + ratio * g.grav[d];
    const double vn = v[d] + g.dt * a;
    P.D(U_V + d, i) = vn;
    P.D(U_W + d, i) = P.D(U_W + d, i) + g.dt * (P.D(U_TCOL + d, i) / I);
    double xn = x[d] + g.dt * vn;
    if (xn >= g.L[d]) xn = xn + (-g.L[d]);
    else if (xn < 0.0) xn = xn + g.L[d];
    P.D(U_X + d, i) = xn;
  }
  P.D(U_ALPHA, i) = af;
}



double eta_of(double e) {
  // ZJS_COLLISION_DEM.F90:30: 3.1415926536 is a single-precision literal
  float pi32 = 3.1415926536f;
  float pi2 = pi32 * pi32;
  return -2 * std::log(e) / std::sqrt((double)pi2 + std::log(e));
}

}  // namespace
}  // namespace ibmdem

using namespace ibmdem;

struct ibmdem_ucase {
  ibmdem_uparams p{};
  UGeom g{};
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err = "ok";
  long long launches = 0;
  int np = 0, cap = 0;
  double* pd = nullptr;
  int* gidx = nullptr;
  uint32_t *kA = nullptr, *vA = nullptr;  // DEM cell of each particle, its slot in the cell
  uint32_t *kC = nullptr, *vC = nullptr;  // fluid cell of each particle, its slot in the cell
  int *demStart = nullptr, *demItems = nullptr, *flStart = nullptr, *flItems = nullptr;
  // per-cell counts of the two cell lists; all zero between steps (the
  // placement zeroes the cells it used), so no sweep clears them
  int *demCount = nullptr, *flCount = nullptr;
  int* nc[2] = {nullptr, nullptr};
  int* partner[2] = {nullptr, nullptr};
  double* xi[2] = {nullptr, nullptr};
  int hcur = 0;
  double* st = nullptr;     // [kStamp * cap] Gaussian stamps in fluid-cell order
  int* occFlag = nullptr;   // [nint + 1] occupied-cell flags, then their exclusive scan
  int* occ = nullptr;       // [min(nint, cap)] occupied fluid cells
  int* nOcc = nullptr;      // their number
  double* T = nullptr;      // [kCellStamp * min(nint, cap)] cell stamps
  float4* pos = nullptr;    // [cap] FP32 positions and radii in DEM-cell order
  int* cstart = nullptr;    // [cap + 1] first flat contact of each particle
  int* owner = nullptr;     // [K * cap] slot of each flat contact
  double* fterm = nullptr;  // [3 * K * cap] per-slot force term
  double* tterm = nullptr;  // [3 * K * cap] per-slot torque term
  int* dTotal = nullptr;    // contacts of the step
  double* alphaf = nullptr;
  double *uf = nullptr, *vf = nullptr, *wf = nullptr;
  int* dErr = nullptr;  // [0] bits, [1] first particle
  // per-phase CUDA-event timing (ibmdem_unresolved_timing_enable)
  bool timing = false;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> spans;
  std::vector<cudaEvent_t> evFree;
  double phaseMs[8] = {};
  long long phaseCount[8] = {};
  int* scan = nullptr;
  bool haveFluid = false, stepped = false;
};

namespace {

int uerr(ibmdem_ucase* u, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (u) u->err = buf;
  return code;
}

#define UCU(call)                                                                             \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) return uerr(u, IBMDEM_ECUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
cudaError_t ualloc(ibmdem_ucase* u, T*& p, size_t n) {
  p = nullptr;
  return cudaMallocAsync(reinterpret_cast<void**>(&p), std::max<size_t>(n, 1) * sizeof(T), u->stream);
}

void ufree_particles(ibmdem_ucase* u) {
  void* ps[] = {u->pd, u->gidx, u->kA, u->vA, u->kC, u->vC, u->demItems, u->flItems,
                u->nc[0], u->nc[1], u->partner[0], u->partner[1], u->xi[0], u->xi[1], u->st, u->pos, u->scan, u->cstart, u->owner,
                u->fterm, u->tterm, u->occFlag, u->occ, u->nOcc, u->T};
  for (void* q : ps)
    if (q) cudaFreeAsync(q, u->stream);
  u->pd = nullptr;
  u->gidx = u->demItems = u->flItems = nullptr;
  u->kA = u->vA = u->kC = u->vC = nullptr;
  u->nc[0] = u->nc[1] = u->partner[0] = u->partner[1] = nullptr;
  u->xi[0] = u->xi[1] = nullptr;
  u->st = nullptr;
  u->pos = nullptr;
  u->cstart = u->owner = nullptr;
  u->fterm = u->tterm = nullptr;
  u->occFlag = u->occ = u->nOcc = nullptr;
  u->T = nullptr;
  u->scan = nullptr;
  u->cap = u->np = 0;
}

int check_errors(ibmdem_ucase* u) {
  int h[2] = {0, 0};
  UCU(cudaMemcpyAsync(h, u->dErr, sizeof h, cudaMemcpyDeviceToHost, u->stream));
  UCU(cudaStreamSynchronize(u->stream));
  if (h[0] & UE_RANGE) return uerr(u, IBMDEM_ERANGE, "particle %d is outside the periodic box", h[1]);
  if (h[0] & UE_CONTACTS)
    return uerr(u, IBMDEM_ECAPACITY, "particle %d touches more than %d partners", h[1], u->g.K);
  return IBMDEM_OK;
}

UPtr uptr(ibmdem_ucase* u) { return UPtr{u->pd, u->gidx, u->cap}; }

enum UPhase : int { UP_LISTS = 0, UP_SEARCH, UP_CONTACTS, UP_STAMPS, UP_ALPHA, UP_DRAG, UP_COUNT };
const char* kUPhaseNames[UP_COUNT] = {"lists", "search", "contacts", "stamps", "alpha", "drag"};

cudaEvent_t take_event(ibmdem_ucase* u) {
  if (!u->evFree.empty()) {
    cudaEvent_t e = u->evFree.back();
    u->evFree.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// CUDA events around one phase on the case's stream when timing is on
struct UScope {
  ibmdem_ucase* u;
  int ph;
  cudaEvent_t a = nullptr;
  UScope(ibmdem_ucase* uu, int p) : u(uu), ph(p) {
    if (!u->timing) return;
    a = take_event(u);
    cudaEventRecord(a, u->stream);
  }
  ~UScope() {
    if (!a) return;
    cudaEvent_t b = take_event(u);
    cudaEventRecord(b, u->stream);
    u->spans.push_back({ph, {a, b}});
  }
};

void collect_timing(ibmdem_ucase* u) {
  cudaStreamSynchronize(u->stream);
  for (auto& sp : u->spans) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, sp.second.first, sp.second.second) == cudaSuccess) {
      u->phaseMs[sp.first] += ms;
      u->phaseCount[sp.first] += 1;
    }
    u->evFree.push_back(sp.second.first);
    u->evFree.push_back(sp.second.second);
  }
  u->spans.clear();
}

int one_step(ibmdem_ucase* u) {
  UGeom& g = u->g;
  cudaStream_t s = u->stream;
  const int np = u->np;
  if (np == 0) return IBMDEM_OK;
  const int nb = nblocks(np);
  UPtr P = uptr(u);
  {
  UScope ts(u, UP_LISTS);
  k_u_keys<<<nb, kBlock, 0, s>>>(g, P, np, u->kA, u->vA, u->demCount, u->kC, u->vC, u->flCount, u->dErr,
                                 u->dErr + 1);
  u->launches++;
  scan_exclusive(u->demCount, u->demStart, g.ncd, nullptr, u->demStart + g.ncd, u->scan, s, &u->launches);
  scan_exclusive(u->flCount, u->flStart, g.nint, nullptr, u->flStart + g.nint, u->scan, s, &u->launches);
  k_u_place<<<nb, kBlock, 0, s>>>(np, u->kA, u->vA, u->demStart, u->demItems, u->demCount);
  k_u_place<<<nb, kBlock, 0, s>>>(np, u->kC, u->vC, u->flStart, u->flItems, u->flCount);
  k_u_order<<<nb, kBlock, 0, s>>>(np, u->kA, u->vA, u->demStart, u->demItems);
  k_u_order<<<nb, kBlock, 0, s>>>(np, u->kC, u->vC, u->flStart, u->flItems);
  u->launches += 4;
  }
  const int o = u->hcur, n = u->hcur ^ 1;
  {
  UScope ts(u, UP_SEARCH);
  k_u_pos32<<<nb, kBlock, 0, s>>>(P, np, u->demItems, u->pos);
  k_u_find<<<nb, kBlock, 0, s>>>(g, P, np, u->demStart, u->demItems, u->pos, u->nc[n], u->partner[n], u->dErr,
                                 u->dErr + 1);
  scan_exclusive(u->nc[n], u->cstart, np, nullptr, u->dTotal, u->scan, s, &u->launches);
  k_u_owner<<<nb, kBlock, 0, s>>>(np, g.K, u->nc[n], u->cstart, u->owner);
  }
  {
  UScope ts(u, UP_CONTACTS);
  k_u_pair<<<gs_blocks((long long)np * g.K), kBlock, 0, s>>>(g, P, u->dTotal, u->owner, u->nc[o], u->partner[o],
                                                            u->xi[o], u->partner[n], u->xi[n], u->fterm, u->tterm);
  k_u_sum<<<nb, kBlock, 0, s>>>(P, np, g.K, u->nc[n], u->fterm, u->tterm);
  }
  {
  UScope ts(u, UP_STAMPS);
  k_u_gauss<<<nb, kBlock, 0, s>>>(g, P, np, u->flItems, u->st);
  }
  {
  UScope ts(u, UP_ALPHA);
  const int nbc = nblocks(g.nint);
  k_u_occ_flag<<<nbc, kBlock, 0, s>>>(g.nint, u->flStart, u->occFlag);
  scan_exclusive(u->occFlag, u->occFlag, g.nint, nullptr, u->nOcc, u->scan, s, &u->launches);
  k_u_occ_list<<<nbc, kBlock, 0, s>>>(g.nint, u->flStart, u->occFlag, u->occ);
  k_u_cellsum<<<gs_blocks(32ll * std::min<long long>(g.nint, np)), kBlock, 0, s>>>(u->nOcc, u->occ, u->flStart,
                                                                                   u->st, u->T);
  k_u_alpha<<<nbc, kBlock, 0, s>>>(g, u->flStart, u->occFlag, u->T, u->alphaf);
  }
  {
  UScope ts(u, UP_DRAG);
  k_u_drag_move<<<nb, kBlock, 0, s>>>(g, P, np, u->uf, u->vf, u->wf, u->alphaf);
  }
  u->launches += 12;
  u->hcur = n;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return uerr(u, IBMDEM_ECUDA, "kernel launch: %s", cudaGetErrorString(e));
  return IBMDEM_OK;
}

}  // namespace

extern "C" {

int ibmdem_unresolved_create(const ibmdem_uparams* p, int32_t device, ibmdem_ucase** out) {
  if (!p || !out) return IBMDEM_EINVAL;
  *out = nullptr;
  if (p->nx < 5 || p->ny < 5 || p->nz < 5 || !(p->dx > 0) || !(p->dcell > 0) || !(p->dt > 0) || !(p->rhof > 0) ||
      !(p->viscf > 0) || p->maxContacts < 1 || !(p->bandwidth > 0) || !(p->ktRatio > 0) || p->mu < 0)
    return IBMDEM_EINVAL;
  if (cudaSetDevice(device) != cudaSuccess) return IBMDEM_ECUDA;
  ibmdem_ucase* u = new (std::nothrow) ibmdem_ucase();
  if (!u) return IBMDEM_ENOMEM;
  u->p = *p;
  u->device = device;
  UGeom& g = u->g;
  g.n[0] = p->nx;
  g.n[1] = p->ny;
  g.n[2] = p->nz;
  g.ni = p->nx + 4;
  g.nj = p->ny + 4;
  g.nint = (long long)p->nx * p->ny * p->nz;
  g.h = p->dx;
  g.vcell = p->dx * p->dx * p->dx;
  g.ncd = 1;
  for (int d = 0; d < 3; ++d) {
    g.L[d] = p->dx * g.n[d];
    g.halfL[d] = 0.5 * g.L[d];
    g.nc[d] = std::max(3, (int)std::floor(g.L[d] / p->dcell));
    g.cs[d] = g.L[d] / g.nc[d];
    g.ncd *= g.nc[d];
    g.grav[d] = p->gravity[d];
  }
  g.K = p->maxContacts;
  g.dt = p->dt;
  g.rhof = p->rhof;
  g.viscf = p->viscf;
  g.knCoeff = p->knCoeff;
  g.knScale = p->knCoeff / (0.1 * p->dx);  // the kn prefactor of every pair
  g.eta = eta_of(p->ResistCoeff);
  g.ktRatio = p->ktRatio;
  g.mu = p->mu;
  g.bandwidth = p->bandwidth;
  g.alphaMin = p->alphaMin;
  if (g.ncd >= (1ll << 31) || g.nint >= (1ll << 31)) {
    delete u;
    return IBMDEM_EUNSUPPORTED;
  }
  const size_t nf = (size_t)g.ni * g.nj * (p->nz + 4);
  cudaError_t e = cudaSuccess;
  auto A = [&](auto& q, size_t n) {
    if (e == cudaSuccess) e = ualloc(u, q, n);
  };
  A(u->uf, nf);
  A(u->vf, nf);
  A(u->wf, nf);
  A(u->alphaf, (size_t)g.nint);
  A(u->demStart, (size_t)g.ncd + 1);
  A(u->flStart, (size_t)g.nint + 1);
  A(u->demCount, (size_t)g.ncd + 1);
  A(u->flCount, (size_t)g.nint + 1);
  A(u->dErr, 2);
  A(u->dTotal, 1);
  if (e == cudaSuccess) {
    cudaMemsetAsync(u->uf, 0, nf * sizeof(double), u->stream);
    cudaMemsetAsync(u->vf, 0, nf * sizeof(double), u->stream);
    cudaMemsetAsync(u->wf, 0, nf * sizeof(double), u->stream);
    cudaMemsetAsync(u->dErr, 0, 2 * sizeof(int), u->stream);
    cudaMemsetAsync(u->demCount, 0, ((size_t)g.ncd + 1) * sizeof(int), u->stream);
    cudaMemsetAsync(u->flCount, 0, ((size_t)g.nint + 1) * sizeof(int), u->stream);
    e = cudaStreamSynchronize(u->stream);
  }
  if (e != cudaSuccess) {
    ibmdem_unresolved_destroy(u);
    return IBMDEM_ENOMEM;
  }
  *out = u;
  return IBMDEM_OK;
}

int ibmdem_unresolved_destroy(ibmdem_ucase* u) {
  if (!u) return IBMDEM_EINVAL;
  cudaSetDevice(u->device);
  cudaStreamSynchronize(u->stream);
  ufree_particles(u);
  void* ps[] = {u->uf, u->vf, u->wf, u->alphaf, u->demStart, u->flStart, u->demCount, u->flCount, u->dErr, u->dTotal};
  for (void* q : ps)
    if (q) cudaFreeAsync(q, u->stream);
  cudaStreamSynchronize(u->stream);
  for (auto& sp : u->spans) {
    cudaEventDestroy(sp.second.first);
    cudaEventDestroy(sp.second.second);
  }
  for (cudaEvent_t e : u->evFree) cudaEventDestroy(e);
  delete u;
  return IBMDEM_OK;
}

const char* ibmdem_unresolved_last_error(const ibmdem_ucase* u) { return u ? u->err.c_str() : "null case"; }

int ibmdem_unresolved_set_stream(ibmdem_ucase* u, void* stream) {
  if (!u) return IBMDEM_EINVAL;
  u->stream = reinterpret_cast<cudaStream_t>(stream);
  return IBMDEM_OK;
}

int64_t ibmdem_unresolved_launch_count(const ibmdem_ucase* u) { return u ? u->launches : 0; }

int ibmdem_unresolved_set_fluid(ibmdem_ucase* u, const double* uf, const double* vf, const double* wf) {
  if (!u || !uf || !vf || !wf) return IBMDEM_EINVAL;
  cudaSetDevice(u->device);
  const size_t nb = sizeof(double) * (size_t)u->g.ni * u->g.nj * (u->p.nz + 4);
  UCU(cudaMemcpyAsync(u->uf, uf, nb, cudaMemcpyHostToDevice, u->stream));
  UCU(cudaMemcpyAsync(u->vf, vf, nb, cudaMemcpyHostToDevice, u->stream));
  UCU(cudaMemcpyAsync(u->wf, wf, nb, cudaMemcpyHostToDevice, u->stream));
  UCU(cudaStreamSynchronize(u->stream));
  u->haveFluid = true;
  return IBMDEM_OK;
}

int ibmdem_unresolved_set_particles(ibmdem_ucase* u, int32_t np, const ibmdem_particle* parts) {
  if (!u || np < 0 || (np > 0 && !parts)) return IBMDEM_EINVAL;
  cudaSetDevice(u->device);
  UCU(cudaStreamSynchronize(u->stream));
  const UGeom& g = u->g;
  for (int i = 0; i < np; ++i)
    for (int d = 0; d < 3; ++d)
      if (!(parts[i].x[d] >= 0.0 && parts[i].x[d] < g.L[d]))
        return uerr(u, IBMDEM_ERANGE, "particle %d is outside the periodic box", i);
  ufree_particles(u);
  // new particles start from clean cell counts
  UCU(cudaMemsetAsync(u->demCount, 0, ((size_t)g.ncd + 1) * sizeof(int), u->stream));
  UCU(cudaMemsetAsync(u->flCount, 0, ((size_t)g.nint + 1) * sizeof(int), u->stream));
  const int cap = std::max(np, 1);
  const size_t K = (size_t)g.K;
  cudaError_t e = cudaSuccess;
  auto A = [&](auto& q, size_t n) {
    if (e == cudaSuccess) e = ualloc(u, q, n);
  };
  A(u->pd, (size_t)U_ND * cap);
  A(u->gidx, (size_t)cap);
  for (auto* q : {&u->kA, &u->vA, &u->kC, &u->vC}) A(*q, (size_t)cap);
  A(u->demItems, (size_t)cap);
  A(u->flItems, (size_t)cap);
  for (int b = 0; b < 2; ++b) {
    A(u->nc[b], (size_t)cap);
    A(u->partner[b], K * cap);
    A(u->xi[b], 3 * K * cap);
  }
  A(u->st, (size_t)kStamp * cap);
  A(u->pos, (size_t)cap);
  A(u->cstart, (size_t)cap + 1);
  const size_t maxOcc = (size_t)std::min<long long>(g.nint, cap);
  A(u->occFlag, (size_t)g.nint + 1);
  A(u->occ, maxOcc);
  A(u->nOcc, 1);
  A(u->T, (size_t)kCellStamp * maxOcc);
  A(u->owner, K * cap);
  A(u->fterm, 3 * K * cap);
  A(u->tterm, 3 * K * cap);
  const long long scanN = std::max<long long>(std::max(g.ncd, g.nint), cap) + 1;
  A(u->scan, (size_t)scan_scratch_ints(scanN));
  if (e != cudaSuccess) {
    ufree_particles(u);
    return uerr(u, IBMDEM_ENOMEM, "particle buffers: %s", cudaGetErrorString(e));
  }
  u->cap = cap;
  u->np = np;
  std::vector<double> hd((size_t)U_ND * cap, 0.0);
  std::vector<int> hg(cap, 0);
  for (int i = 0; i < np; ++i) {
    const ibmdem_particle& q = parts[i];
    auto put = [&](int f, double v) { hd[(size_t)f * cap + i] = v; };
    put(U_RAD, q.rad);
    put(U_RHO, q.rho);
    put(U_VOL, q.vol);
    put(U_M, q.m);
    put(U_I, q.I);
    for (int d = 0; d < 3; ++d) {
      put(U_X + d, q.x[d]);
      put(U_V + d, q.v[d]);
      put(U_W + d, q.omega[d]);
      put(U_FCOL + d, q.fcol[d]);
      put(U_TCOL + d, q.tcol[d]);
      put(U_FDRAG + d, q.fdrag[d]);
    }
    put(U_ALPHA, q.alphaf);
    hg[i] = q.globalIdx;
  }
  UCU(cudaMemcpyAsync(u->pd, hd.data(), sizeof(double) * hd.size(), cudaMemcpyHostToDevice, u->stream));
  UCU(cudaMemcpyAsync(u->gidx, hg.data(), sizeof(int) * hg.size(), cudaMemcpyHostToDevice, u->stream));
  UCU(cudaMemsetAsync(u->nc[0], 0, sizeof(int) * cap, u->stream));
  UCU(cudaMemsetAsync(u->nc[1], 0, sizeof(int) * cap, u->stream));
  UCU(cudaMemsetAsync(u->dErr, 0, 2 * sizeof(int), u->stream));
  UCU(cudaStreamSynchronize(u->stream));
  u->hcur = 0;
  u->stepped = false;
  return IBMDEM_OK;
}

int ibmdem_unresolved_get_particles(ibmdem_ucase* u, ibmdem_particle* parts, int32_t cap, int32_t* n) {
  if (!u) return IBMDEM_EINVAL;
  cudaSetDevice(u->device);
  int rc = check_errors(u);
  if (rc) return rc;
  if (n) *n = u->np;
  if (!parts || u->np == 0) return IBMDEM_OK;
  std::vector<double> hd((size_t)U_ND * u->cap);
  std::vector<int> hg(u->cap);
  UCU(cudaMemcpyAsync(hd.data(), u->pd, sizeof(double) * hd.size(), cudaMemcpyDeviceToHost, u->stream));
  UCU(cudaMemcpyAsync(hg.data(), u->gidx, sizeof(int) * hg.size(), cudaMemcpyDeviceToHost, u->stream));
  UCU(cudaStreamSynchronize(u->stream));
  const int m = std::min(cap, u->np);
  for (int i = 0; i < m; ++i) {
    ibmdem_particle& q = parts[i];
    std::memset(&q, 0, sizeof q);
    auto get = [&](int f) { return hd[(size_t)f * u->cap + i]; };
    q.globalIdx = hg[i];
    q.rad = get(U_RAD);
    q.rho = get(U_RHO);
    q.vol = get(U_VOL);
    q.m = get(U_M);
    q.I = get(U_I);
    for (int d = 0; d < 3; ++d) {
      q.x[d] = get(U_X + d);
      q.v[d] = get(U_V + d);
      q.omega[d] = get(U_W + d);
      q.fcol[d] = get(U_FCOL + d);
      q.tcol[d] = get(U_TCOL + d);
      q.fdrag[d] = get(U_FDRAG + d);
    }
    q.alphaf = get(U_ALPHA);
  }
  return IBMDEM_OK;
}

int ibmdem_unresolved_get_volume_fraction(ibmdem_ucase* u, double* alphaf) {
  if (!u || !alphaf) return IBMDEM_EINVAL;
  cudaSetDevice(u->device);
  int rc = check_errors(u);
  if (rc) return rc;
  if (!u->stepped) return uerr(u, IBMDEM_ESTATE, "no step has run");
  UCU(cudaMemcpyAsync(alphaf, u->alphaf, sizeof(double) * u->g.nint, cudaMemcpyDeviceToHost, u->stream));
  UCU(cudaStreamSynchronize(u->stream));
  return IBMDEM_OK;
}

int ibmdem_unresolved_get_contacts(ibmdem_ucase* u, int32_t* start, int32_t* partner, double* xi,
                                   int32_t* ncontacts) {
  if (!u) return IBMDEM_EINVAL;
  cudaSetDevice(u->device);
  int rc = check_errors(u);
  if (rc) return rc;
  const int np = u->np, K = u->g.K, b = u->hcur;
  std::vector<int> nc(std::max(np, 1), 0), pa((size_t)K * std::max(np, 1));
  std::vector<double> xv;
  if (np) {
    UCU(cudaMemcpyAsync(nc.data(), u->nc[b], sizeof(int) * np, cudaMemcpyDeviceToHost, u->stream));
    UCU(cudaMemcpyAsync(pa.data(), u->partner[b], sizeof(int) * (size_t)K * np, cudaMemcpyDeviceToHost, u->stream));
    if (xi) {
      xv.resize((size_t)3 * K * np);
      UCU(cudaMemcpyAsync(xv.data(), u->xi[b], sizeof(double) * xv.size(), cudaMemcpyDeviceToHost, u->stream));
    }
    UCU(cudaStreamSynchronize(u->stream));
  }
  int tot = 0;
  for (int i = 0; i < np; ++i) {
    if (start) start[i] = tot;
    for (int s = 0; s < nc[i]; ++s) {
      if (partner) partner[tot] = pa[(size_t)i * K + s];
      if (xi)
        for (int d = 0; d < 3; ++d) xi[3 * (size_t)tot + d] = xv[((size_t)i * K + s) * 3 + d];
      ++tot;
    }
  }
  if (start) start[np] = tot;
  if (ncontacts) *ncontacts = tot;
  return IBMDEM_OK;
}

int ibmdem_unresolved_step(ibmdem_ucase* u, int32_t nsteps) {
  if (!u || nsteps < 0) return IBMDEM_EINVAL;
  if (cudaSetDevice(u->device) != cudaSuccess) return uerr(u, IBMDEM_ECUDA, "cudaSetDevice failed");
  if (!u->haveFluid) return uerr(u, IBMDEM_ESTATE, "no fluid field");
  for (int s = 0; s < nsteps; ++s) {
    int rc = one_step(u);
    if (rc) return rc;
    u->stepped = true;
  }
  return IBMDEM_OK;
}

int ibmdem_unresolved_timing_enable(ibmdem_ucase* u, int32_t on) {
  if (!u) return IBMDEM_EINVAL;
  u->timing = on != 0;
  return IBMDEM_OK;
}

int ibmdem_unresolved_get_timing(ibmdem_ucase* u, double* ms, int64_t* counts, int32_t n, int32_t reset) {
  if (!u) return IBMDEM_EINVAL;
  collect_timing(u);
  for (int i = 0; i < n && i < UP_COUNT; ++i) {
    if (ms) ms[i] = u->phaseMs[i];
    if (counts) counts[i] = u->phaseCount[i];
  }
  if (reset)
    for (int i = 0; i < UP_COUNT; ++i) {
      u->phaseMs[i] = 0.0;
      u->phaseCount[i] = 0;
    }
  return UP_COUNT;
}

const char* ibmdem_unresolved_phase_name(int32_t i) { return (i >= 0 && i < UP_COUNT) ? kUPhaseNames[i] : ""; }

int ibmdem_unresolved_synchronize(ibmdem_ucase* u) {
  if (!u) return IBMDEM_EINVAL;
  cudaSetDevice(u->device);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return uerr(u, IBMDEM_ECUDA, "%s", cudaGetErrorString(e));
  return check_errors(u);
}

int ibmdem_CalculateDragForce(int32_t n, const double* rho, const double* rad, const double* v, double denf,
                              const double* alphaf, const double* velf, double* beta, void* stream) {
  if (n < 0 || (n > 0 && (!rho || !rad || !v || !alphaf || !velf || !beta)) || !(denf > 0)) return IBMDEM_EINVAL;
  if (n == 0) return IBMDEM_OK;
  k_drag_beta<<<nblocks(n), kBlock, 0, reinterpret_cast<cudaStream_t>(stream)>>>(n, rho, rad, v, denf, alphaf, velf,
                                                                                 beta);
  return cudaGetLastError() == cudaSuccess ? IBMDEM_OK : IBMDEM_ECUDA;
}

}  // extern "C"
