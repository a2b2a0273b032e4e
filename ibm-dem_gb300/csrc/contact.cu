// contact.cu — RebuildParcelCollisionListDEM (ZJS_UPDATE_LIST_DEM.F90:248-286)
// and CalculateCollisionForce (ZJS_COLLISION_DEM.F90:21-74).
//
// The reference scans, for every local parcel, the 125 cells around its cell
// and every parcel in them.  Parcels of one body never pair (MSIdx test), so a
// body-level broad phase removes almost all of that work: a parcel can only
// have a partner when some other body's bounding sphere, grown by the contact
// cut-off plus a margin far above FP32 rounding, reaches it.  Parcels that pass
// this conservative filter run the reference scan unchanged (same cells, same
// order, same FP64 predicate), so the lists are identical, in order, to the
// reference's; the others provably have empty lists.
#include "common.cuh"
#include "kernels.cuh"
#include "prims.cuh"

namespace ibmdem {

namespace {

// minimum-image difference (body centres are not wrapped and may drift)
__device__ inline float min_image_f(float d, float L) { return d - L * rintf(d / L); }

__global__ void k_body_bound(Recs R, Geom g, const Counters* cnt, const ibmdem_multisphere* B, int nMS,
                             unsigned* r2bits) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  int b = -1;
  unsigned v = 0u;  // squared distance as float bits (non-negative: the order is the integer order)
  if (m < cnt->npLocal) {
    b = R.I(I_MSIDX, m) - 1;
    if (b >= 0 && b < nMS) {
      float d2 = 0.f;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        float dd = min_image_f((float)R.D(D_X + d, m) - (float)B[b].x[d], (float)g.len[d]);
        d2 += dd * dd;
      }
      v = __float_as_uint(d2);
    } else {
      b = -1;
    }
  }
  // a body's markers are mostly neighbours in part order: maximum over each run
  // of equal bodies in the warp, one atomic per run
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned vo = __shfl_up_sync(0xffffffffu, v, o);
    const int bo = __shfl_up_sync(0xffffffffu, b, o);
    if (lane >= o && bo == b) v = max(v, vo);
  }
  const int next = __shfl_down_sync(0xffffffffu, b, 1);
  if (b >= 0 && (lane == 31 || next != b)) atomicMax(&r2bits[b], v);
}

__global__ void k_body_pairs(const ibmdem_multisphere* B, int nMS, Geom g, const unsigned* r2bits, float reach,
                             int* partnerCnt, int* partners, int maxPartners, Counters* cnt) {
  int a = blockIdx.y;
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= nMS || b >= nMS || b <= a) return;
  float d2 = 0.f;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    float dd = min_image_f((float)B[a].x[d] - (float)B[b].x[d], (float)g.len[d]);
    d2 += dd * dd;
  }
  float lim = sqrtf(__uint_as_float(r2bits[a])) + sqrtf(__uint_as_float(r2bits[b])) + reach;
  if (d2 < lim * lim) {
    int qa = atomicAdd(&partnerCnt[a], 1);
    int qb = atomicAdd(&partnerCnt[b], 1);
    if (qa < maxPartners) partners[a * maxPartners + qa] = b;
    else set_err(cnt, E_PARTNER, a);
    if (qb < maxPartners) partners[b * maxPartners + qb] = a;
    else set_err(cnt, E_PARTNER, b);
  }
}

__global__ void k_marker_active(Recs R, Geom g, const Counters* cnt, const ibmdem_multisphere* B, int nMS,
                                const unsigned* r2bits, const int* partnerCnt, const int* partners,
                                int maxPartners, float reach, int* flag) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= cnt->npLocal) return;
  int b = R.I(I_MSIDX, m) - 1;
  int act = 0;
  if (b >= 0 && b < nMS) {
    int np = min(partnerCnt[b], maxPartners);
    float x[3] = {(float)R.D(D_X, m), (float)R.D(D_X + 1, m), (float)R.D(D_X + 2, m)};
    for (int q = 0; q < np && !act; ++q) {
      int o = partners[b * maxPartners + q];
      float d2 = 0.f;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        float dd = min_image_f(x[d] - (float)B[o].x[d], (float)g.len[d]);
        d2 += dd * dd;
      }
      float lim = sqrtf(__uint_as_float(r2bits[o])) + reach;
      act = d2 < lim * lim;
    }
  }
  flag[m] = act;
}

__global__ void k_compact_active(const Counters* cnt, const int* flag, const int* pos, int* list) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= cnt->npLocal || !flag[m]) return;
  list[pos[m]] = m;
}

// Collision (ZJS_COLLISION_DEM.F90:2-19) inside the 125-cell scan of
// RebuildParcelCollisionListDEM, one warp per candidate parcel: in each round
// the 32 lanes take 32 consecutive stencil cells (kk, jj, ii order), count
// their hits, and a warp prefix places them, so the list keeps the reference's
// order (stencil cell, then the cell's part order).  FILL = false counts.
// A partner must have pType -1 (ZJS_UPDATE_LIST_DEM.F90:272): images made
// across a solid wall (pType 1) never are.
__device__ inline bool partner_type_ok(const Geom& g, const Counters* cnt, const int* imgShift, int j) {
  if (!g.anyWall) return true;
  const int q = j - cnt->npLocal;
  return q < 0 || !((imgShift[q] >> kWallImgBit) & 1);
}

template <bool FILL>
__global__ void k_pair_scan(Recs R, Geom g, const Counters* cnt, const int* activeList, const int* nActive,
                            const int* cellStart, const int* cellItems, const int* imgShift, int* pairCnt,
                            const int* pairStart, int* pairIdx, long long capPairs, Counters* cntw) {
  const int lane = threadIdx.x & 31;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const int na = *nActive;
  for (long long q = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < na; q += nw) {
    const int ii = activeList[q];
    int ci, cj, ck;
    cell_coords(g, R.I(I_CELL, ii), ci, cj, ck);
    const int msi = R.I(I_MSIDX, ii);
    const double xi0 = R.D(D_X, ii), xi1 = R.D(D_X + 1, ii), xi2 = R.D(D_X + 2, ii);
    const long long base = FILL ? pairStart[ii] : 0;
    int total = 0;
    for (int round = 0; round < 4; ++round) {
      const int jst = round * 32 + lane;
      int s = 0, e = 0;
      if (jst < 125) {
        const int a = ci + jst % 5 - 2, b = cj + (jst / 5) % 5 - 2, c = ck + jst / 25 - 2;
        if (a >= -1 && a <= g.n[0] + 2 && b >= -1 && b <= g.n[1] + 2 && c >= -1 && c <= g.n[2] + 2) {
          const int cell = cell_id(g, a, b, c);
          s = cellStart[cell - 1];
          e = cellStart[cell];
        }
      }
      int mine = 0;
      for (int k = s; k < e; ++k) {
        const int jjx = cellItems[k];
        if (R.I(I_MSIDX, jjx) == msi) continue;
        const double xij1 = xi0 - R.D(D_X, jjx);
        const double xij2 = xi1 - R.D(D_X + 1, jjx);
        const double xij3 = xi2 - R.D(D_X + 2, jjx);
        const double distSqr = xij1 * xij1 + xij2 * xij2 + xij3 * xij3;
        if (distSqr < g.cut2 && jjx != ii && partner_type_ok(g, cnt, imgShift, jjx)) ++mine;
      }
      int x = mine;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      if (FILL && mine) {
        long long at = base + total + x - mine;
        for (int k = s; k < e; ++k) {
          const int jjx = cellItems[k];
          if (R.I(I_MSIDX, jjx) == msi) continue;
          const double xij1 = xi0 - R.D(D_X, jjx);
          const double xij2 = xi1 - R.D(D_X + 1, jjx);
          const double xij3 = xi2 - R.D(D_X + 2, jjx);
          const double distSqr = xij1 * xij1 + xij2 * xij2 + xij3 * xij3;
          if (distSqr < g.cut2 && jjx != ii && partner_type_ok(g, cnt, imgShift, jjx)) {
            if (at < capPairs) pairIdx[at] = jjx;
            else set_err(cntw, E_PAIRCAP, (int)at);
            ++at;
          }
        }
      }
      total += __shfl_sync(0xffffffffu, x, 31);
    }
    if (!FILL && lane == 0) pairCnt[ii] = total;
  }
}

__global__ void k_set_pair_total(Counters* cnt, const int* total, long long capPairs) {
  int n = *total;
  if (n > capPairs) {
    atomicOr(&cnt->err, E_PAIRCAP);
    cnt->errInfo = n;
  }
  cnt->nPairs = n;
}

// CalculateCollisionForce (ZJS_COLLISION_DEM.F90:21-74), one thread per local
__global__ void k_collision_force(Recs R, Geom g, const Counters* cnt, const int* pairStart, const int* pairIdx,
                                  long long capPairs) {
  int ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= cnt->npLocal) return;
  double fc1 = 0, fc2 = 0, fc3 = 0;
  int s = pairStart[ii], e = pairStart[ii + 1];
  if (e > capPairs) e = (int)capPairs;
  if (s < e) {
    const double xi0 = R.D(D_X, ii), xi1 = R.D(D_X + 1, ii), xi2 = R.D(D_X + 2, ii);
    const double vi0 = R.D(D_V, ii), vi1 = R.D(D_V + 1, ii), vi2 = R.D(D_V + 2, ii);
    const double mi = R.D(D_M, ii), ri = R.D(D_RADEFF, ii);
    for (int q = s; q < e; ++q) {
      int j = pairIdx[q];
      double r1 = xi0 - R.D(D_X, j);
      double r2 = xi1 - R.D(D_X + 1, j);
      double r3 = xi2 - R.D(D_X + 2, j);
      double dist = sqrt(r1 * r1 + r2 * r2 + r3 * r3);
      double n1 = r1 / dist, n2 = r2 / dist, n3 = r3 / dist;
      double mj = R.D(D_M, j);
      double meff = 2 * mi * mj / (mi + mj);
      double rij = ri + R.D(D_RADEFF, j);
      double deltan = rij - dist;
      double kn = g.knCoeff / (0.1 * g.di) * meff;
      double etan = g.eta * sqrt(meff * kn);
      double f1 = 0, f2 = 0, f3 = 0;
      double vnij = n1 * (vi0 - R.D(D_V, j)) + n2 * (vi1 - R.D(D_V + 1, j)) + n3 * (vi2 - R.D(D_V + 2, j));
      if (deltan > 0) {
        f1 = n1 * (kn * deltan - etan * vnij);
        f2 = n2 * (kn * deltan - etan * vnij);
        f3 = n3 * (kn * deltan - etan * vnij);
      }
      fc1 = fc1 + f1;
      fc2 = fc2 + f2;
      fc3 = fc3 + f3;
    }
  }
  R.D(D_FCOL, ii) = fc1;
  R.D(D_FCOL + 1, ii) = fc2;
  R.D(D_FCOL + 2, ii) = fc3;
}

// The pair forces with tangential friction (ibmdem_set_friction; the
// reference's law is normal only).  The normal part is the law above, term by
// term.  For a touching pair (deltan > 0), with u = v_i - v_j the relative
// marker velocity (marker velocities carry their body's rotation):
//   vt = u - vn n;  h = the pair's tangential displacement of the last call
//   (found by the partner's persistent parcel id, I_PID; 0 for a new contact), projected on the
//   tangent plane, plus dtDEM vt;  kt = ktRatio kn, etat = eta sqrt(meff kt),
//   ft = -kt h - etat vt, scaled to mu |fn| beyond the Coulomb limit (h then
//   the sliding value -(ft + etat vt) / kt);  fcol_i += n fn + ft.
// One thread per local; the history is read from one side and written to the
// other (k_hist_finish flips the side and maps the parcel ids to the locals).
__global__ void k_collision_force_friction(Recs R, Geom g, const Counters* cnt, const int* pairStart,
                                           const int* pairIdx, long long capPairs, double ktRatio, double mu,
                                           int2* range0, int2* range1, int* gid0, int* gid1, double* xs0,
                                           double* xs1, const int* pidMap, int nPid) {
  const int ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii >= cnt->npLocal) return;
  const int side = cnt->histSide;
  const int2* oRange = side ? range1 : range0;
  const int* oGid = side ? gid1 : gid0;
  const double* oXi = side ? xs1 : xs0;
  int2* nRange = side ? range0 : range1;
  int* nGid = side ? gid0 : gid1;
  double* nXi = side ? xs0 : xs1;
  double fc1 = 0, fc2 = 0, fc3 = 0;
  int s = pairStart[ii], e = pairStart[ii + 1];
  if (e > capPairs) e = (int)capPairs;
  if (s > e) s = e;
  nRange[ii] = make_int2(s, e);
  const int pi = R.I(I_PID, ii);
  const int o = (pi >= 0 && pi < nPid) ? pidMap[pi] : -1;
  const int2 orr = o >= 0 ? oRange[o] : make_int2(0, 0);
  if (s < e) {
    const double xi0 = R.D(D_X, ii), xi1 = R.D(D_X + 1, ii), xi2 = R.D(D_X + 2, ii);
    const double vi0 = R.D(D_V, ii), vi1 = R.D(D_V + 1, ii), vi2 = R.D(D_V + 2, ii);
    const double mi = R.D(D_M, ii), ri = R.D(D_RADEFF, ii);
    for (int q = s; q < e; ++q) {
      int j = pairIdx[q];
      double r1 = xi0 - R.D(D_X, j);
      double r2 = xi1 - R.D(D_X + 1, j);
      double r3 = xi2 - R.D(D_X + 2, j);
      double dist = sqrt(r1 * r1 + r2 * r2 + r3 * r3);
      double n1 = r1 / dist, n2 = r2 / dist, n3 = r3 / dist;
      double mj = R.D(D_M, j);
      double meff = 2 * mi * mj / (mi + mj);
      double rij = ri + R.D(D_RADEFF, j);
      double deltan = rij - dist;
      double kn = g.knCoeff / (0.1 * g.di) * meff;
      double etan = g.eta * sqrt(meff * kn);
      double f1 = 0, f2 = 0, f3 = 0;
      double u1 = vi0 - R.D(D_V, j), u2 = vi1 - R.D(D_V + 1, j), u3 = vi2 - R.D(D_V + 2, j);
      double vnij = n1 * u1 + n2 * u2 + n3 * u3;
      double h1 = 0, h2 = 0, h3 = 0;
      int hg = -1;
      if (deltan > 0) {
        const int gj = R.I(I_PID, j);
        double fn = kn * deltan - etan * vnij;
        double vt1 = u1 - vnij * n1, vt2 = u2 - vnij * n2, vt3 = u3 - vnij * n3;
        for (int t = orr.x; t < orr.y; ++t)
          if (oGid[t] == gj) {
            h1 = oXi[3 * (size_t)t];
            h2 = oXi[3 * (size_t)t + 1];
            h3 = oXi[3 * (size_t)t + 2];
            break;
          }
        double hn = n1 * h1 + n2 * h2 + n3 * h3;
        h1 = h1 - hn * n1;
        h2 = h2 - hn * n2;
        h3 = h3 - hn * n3;
        h1 = h1 + g.dtDEM * vt1;
        h2 = h2 + g.dtDEM * vt2;
        h3 = h3 + g.dtDEM * vt3;
        double kt = ktRatio * kn;
        double etat = g.eta * sqrt(meff * kt);
        double ft1 = -kt * h1 - etat * vt1, ft2 = -kt * h2 - etat * vt2, ft3 = -kt * h3 - etat * vt3;
        double ftm = sqrt(ft1 * ft1 + ft2 * ft2 + ft3 * ft3);
        double lim = mu * fabs(fn);
        if (ftm > lim) {
          double sc = lim / ftm;
          ft1 = ft1 * sc;
          ft2 = ft2 * sc;
          ft3 = ft3 * sc;
          h1 = -(ft1 + etat * vt1) / kt;
          h2 = -(ft2 + etat * vt2) / kt;
          h3 = -(ft3 + etat * vt3) / kt;
        }
        f1 = n1 * fn + ft1;
        f2 = n2 * fn + ft2;
        f3 = n3 * fn + ft3;
        hg = gj;
      }
      nGid[q] = hg;
      nXi[3 * (size_t)q] = h1;
      nXi[3 * (size_t)q + 1] = h2;
      nXi[3 * (size_t)q + 2] = h3;
      fc1 = fc1 + f1;
      fc2 = fc2 + f2;
      fc3 = fc3 + f3;
    }
  }
  R.D(D_FCOL, ii) = fc1;
  R.D(D_FCOL + 1, ii) = fc2;
  R.D(D_FCOL + 2, ii) = fc3;
}

// after the friction forces: parcel id -> local of this call, and the side flips
__global__ void k_hist_finish(Recs R, Counters* cnt, int* pidMap, int nPid) {
  const int ii = blockIdx.x * blockDim.x + threadIdx.x;
  if (ii == 0) cnt->histSide ^= 1;
  if (ii >= cnt->npLocal) return;
  const int pi = R.I(I_PID, ii);
  if (pi >= 0 && pi < nPid) pidMap[pi] = ii;
}

// ---- CalculateSolidBoundaryCollisionForce (ZJS_COLLISION_DEM.F90:76-148) ----
// plane of face f (0..5 = -x,+x,-y,+y,-z,+z): pointBound and normBound
// (ZJS_INIT_DEM.F90:120-137)
struct WallHit {
  double dist, cp1, cp2, cp3, kn, deltan;
  double n1, n2, n3;
};
__device__ inline WallHit wall_contact(const Geom& g, int f, double x1, double x2, double x3, double m,
                                       double radeff) {
  WallHit w;
  const int d = f >> 1;
  const bool hi = f & 1;
  const double p1 = hi ? g.end[0] : g.start[0], p2 = hi ? g.end[1] : g.start[1], p3 = hi ? g.end[2] : g.start[2];
  const double s = hi ? -1.0 : 1.0;
  w.n1 = d == 0 ? s : 0.0;
  w.n2 = d == 1 ? s : 0.0;
  w.n3 = d == 2 ? s : 0.0;
  const double r1 = x1 - p1, r2 = x2 - p2, r3 = x3 - p3;
  w.dist = r1 * w.n1 + r2 * w.n2 + r3 * w.n3;
  w.cp1 = x1 - w.dist * w.n1;
  w.cp2 = x2 - w.dist * w.n2;
  w.cp3 = x3 - w.dist * w.n3;
  w.deltan = radeff - w.dist;
  w.kn = g.knCoeff / (0.1 * g.di) * m;
  return w;
}

// Local parcels in the first or last interior cell layer feel every solid
// wall, faces in order, after their pair forces; flag marks the parcels with a
// wall contact (for the probe sums).
__global__ void k_wall_force(Recs R, Geom g, const Counters* cnt, int* flag) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= cnt->npLocal) return;
  int a, b, cc;
  cell_coords(g, R.I(I_CELL, m), a, b, cc);
  int hit = 0;
  if (a == 1 || a == g.n[0] || b == 1 || b == g.n[1] || cc == 1 || cc == g.n[2]) {
    const double x1 = R.D(D_X, m), x2 = R.D(D_X + 1, m), x3 = R.D(D_X + 2, m);
    const double v1 = R.D(D_V, m), v2 = R.D(D_V + 1, m), v3 = R.D(D_V + 2, m);
    const double meff = R.D(D_M, m), rij = R.D(D_RADEFF, m);
    double fc1 = R.D(D_FCOL, m), fc2 = R.D(D_FCOL + 1, m), fc3 = R.D(D_FCOL + 2, m);
    for (int f = 0; f < 6; ++f) {
      if (!g.wall[f >> 1]) continue;
      const WallHit w = wall_contact(g, f, x1, x2, x3, meff, rij);
      const double etan = g.eta * sqrt(meff * w.kn);
      const double vnij = w.n1 * v1 + w.n2 * v2 + w.n3 * v3;
      if (w.deltan > 0) {
        fc1 = fc1 + w.n1 * (w.kn * w.deltan - etan * vnij);
        fc2 = fc2 + w.n2 * (w.kn * w.deltan - etan * vnij);
        fc3 = fc3 + w.n3 * (w.kn * w.deltan - etan * vnij);
        hit = 1;
      }
    }
    R.D(D_FCOL, m) = fc1;
    R.D(D_FCOL + 1, m) = fc2;
    R.D(D_FCOL + 2, m) = fc3;
  }
  if (flag) flag[m] = hit;
}

__global__ void k_wall_list(const Counters* cnt, const int* flag, const int* pos, int* list) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m < cnt->npLocal && flag[m]) list[pos[m]] = m;
}

// WallProbeCollision (ZJS_COLLISION_DEM.F90:150-179); a NaN angle sum counts as
// inside, as the reference's comparison is false for it
__device__ inline bool probe_contains(const ibmdem_wall_probe& pr, double cp1, double cp2, double cp3) {
  double theta = 0.0;
  for (int q = 0; q < 4; ++q) {
    const int qj = q + 1 > 3 ? q + 1 - 4 : q + 1;
    const double ni1 = pr.points[q][0] - cp1, ni2 = pr.points[q][1] - cp2, ni3 = pr.points[q][2] - cp3;
    const double nj1 = pr.points[qj][0] - cp1, nj2 = pr.points[qj][1] - cp2, nj3 = pr.points[qj][2] - cp3;
    double t = (ni1 * nj1 + ni2 * nj2 + ni3 * nj3) /
               (sqrt(ni1 * ni1 + ni2 * ni2 + ni3 * ni3) * sqrt(nj1 * nj1 + nj2 * nj2 + nj3 * nj3));
    theta = theta + acos(t);
  }
  const double pi = acos(-1.0);
  return !(fabs(theta - 2 * pi) > 0.001 * pi);
}

// one thread per probe: the normal spring forces of the listed parcels whose
// contact point on the probe's face lies inside it, in part order
__global__ void k_probe_sum(Recs R, Geom g, const int* list, const int* nList, ibmdem_wall_probe* probes, int nProbe) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nProbe) return;
  ibmdem_wall_probe pr = probes[q];
  const int f = pr.face - 1;
  double s1 = 0.0, s2 = 0.0, s3 = 0.0;
  const int n = *nList;
  for (int t = 0; t < n; ++t) {
    const int m = list[t];
    const WallHit w = wall_contact(g, f, R.D(D_X, m), R.D(D_X + 1, m), R.D(D_X + 2, m), R.D(D_M, m),
                                   R.D(D_RADEFF, m));
    if (!(w.deltan > 0)) continue;
    if (!probe_contains(pr, w.cp1, w.cp2, w.cp3)) continue;
    s1 = s1 + w.n1 * w.kn * w.deltan;
    s2 = s2 + w.n2 * w.kn * w.deltan;
    s3 = s3 + w.n3 * w.kn * w.deltan;
  }
  probes[q].force[0] = s1;
  probes[q].force[1] = s2;
  probes[q].force[2] = s3;
}

}  // namespace

void launch_wall_force(Ctx& c) {
  if (!c.g.anyWall) return;
  cudaStream_t s = c.stream;
  const int nbl = nblocks(c.capLocal);
  const bool probes = c.nProbe > 0;
  k_wall_force<<<nbl, kBlock, 0, s>>>(c.rec(), c.g, c.dCnt, probes ? c.iTmpA : nullptr);
  c.launches++;
  if (!probes) return;
  // the contact lists are built, so their scratch (iTmpA/B, activeList) is free here
  scan_exclusive(c.iTmpA, c.iTmpB, c.capLocal, &c.dCnt->npLocal, c.dTotal + 3, c.scanScratch, s, &c.launches);
  k_wall_list<<<nbl, kBlock, 0, s>>>(c.dCnt, c.iTmpA, c.iTmpB, c.activeList);
  k_probe_sum<<<1, 64, 0, s>>>(c.rec(), c.g, c.activeList, c.dTotal + 3, c.dProbes, c.nProbe);
  c.launches += 2;
}

void rebuild_collision_lists(Ctx& c) {
  cudaStream_t s = c.stream;
  const int nbl = nblocks(c.capLocal);
  // conservative reach: contact cut-off plus a margin far above FP32 error
  float hmax = (float)fmax(c.g.h[0], fmax(c.g.h[1], c.g.h[2]));
  float reach = (float)sqrt(c.g.cut2) + 0.05f * hmax + 1e-5f * (float)fmax(c.g.len[0], fmax(c.g.len[1], c.g.len[2]));
  if (c.nMS > 0) {
    cudaMemsetAsync(c.bodyR2, 0, sizeof(unsigned) * c.nMS, s);
    cudaMemsetAsync(c.partnerCnt, 0, sizeof(int) * c.nMS, s);
    k_body_bound<<<nbl, kBlock, 0, s>>>(c.rec(), c.g, c.dCnt, c.dBodies, c.nMS, c.bodyR2);
    dim3 grid(nblocks(c.nMS), c.nMS);
    k_body_pairs<<<grid, kBlock, 0, s>>>(c.dBodies, c.nMS, c.g, c.bodyR2, reach, c.partnerCnt, c.partners,
                                         c.maxPartners, c.dCnt);
    k_marker_active<<<nbl, kBlock, 0, s>>>(c.rec(), c.g, c.dCnt, c.dBodies, c.nMS, c.bodyR2, c.partnerCnt,
                                           c.partners, c.maxPartners, reach, c.iTmpA);
    c.launches += 3;
  } else {
    cudaMemsetAsync(c.iTmpA, 0, sizeof(int) * c.capLocal, s);
  }
  scan_exclusive(c.iTmpA, c.iTmpB, c.capLocal, &c.dCnt->npLocal, &c.dCnt->nActive, c.scanScratch, s, &c.launches);
  k_compact_active<<<nbl, kBlock, 0, s>>>(c.dCnt, c.iTmpA, c.iTmpB, c.activeList);
  cudaMemsetAsync(c.pairCnt, 0, sizeof(int) * (c.capLocal + 1), s);
  const int nbw = gs_blocks(32ll * c.capLocal);
  k_pair_scan<false><<<nbw, kBlock, 0, s>>>(c.rec(), c.g, c.dCnt, c.activeList, &c.dCnt->nActive, c.cellStart,
                                            c.cellItems, c.imgShift, c.pairCnt, nullptr, nullptr, c.capPairs,
                                            c.dCnt);
  scan_exclusive(c.pairCnt, c.pairStart, c.capLocal + 1, nullptr, c.dTotal, c.scanScratch, s, &c.launches);
  k_set_pair_total<<<1, 1, 0, s>>>(c.dCnt, c.dTotal, c.capPairs);
  k_pair_scan<true><<<nbw, kBlock, 0, s>>>(c.rec(), c.g, c.dCnt, c.activeList, &c.dCnt->nActive, c.cellStart,
                                           c.cellItems, c.imgShift, c.pairCnt, c.pairStart, c.pairIdx, c.capPairs,
                                           c.dCnt);
  c.launches += 4;
}

void launch_collision_force(Ctx& c) {
  if (c.ktRatio > 0.0 && c.pidMap) {
    k_collision_force_friction<<<nblocks(c.capLocal), kBlock, 0, c.stream>>>(
        c.rec(), c.g, c.dCnt, c.pairStart, c.pairIdx, c.capPairs, c.ktRatio, c.mu, c.histRange[0], c.histRange[1],
        c.histGid[0], c.histGid[1], c.histXi[0], c.histXi[1], c.pidMap, c.capLocal);
    k_hist_finish<<<nblocks(c.capLocal), kBlock, 0, c.stream>>>(c.rec(), c.dCnt, c.pidMap, c.capLocal);
    c.launches += 2;
    return;
  }
  k_collision_force<<<nblocks(c.capLocal), kBlock, 0, c.stream>>>(c.rec(), c.g, c.dCnt, c.pairStart, c.pairIdx,
                                                                  c.capPairs);
  c.launches++;
}

}  // namespace ibmdem
