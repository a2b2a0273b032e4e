// ibm.cu — immersed-boundary interpolation, direct forcing and spreading.
//
// Reference: UpdateLocal/GhostCellWeightListDEM (ZJS_UPDATE_LIST_DEM.F90:323-416)
// with GetWeight / DeltaFunction3D (ZJS_INTERPOLATE_DEM.F90:2-17,
// interpolation.F90:2-33), UpdateFluidVelocityOnLagrangianPoints and
// UpdateMomentumSourceTerm (ZJS_VOLUMEFRACTION_DEM.F90:2-67), VelocityPostGuess
// (fluid.F90:135-153) and the periodic halo refill (boundary.F90:122-147).
//
// The reference evaluates the 3-point delta kernel on all 125 stencil cells.
// Per axis at most three nodes have a non-zero weight: the unshifted kernel is
// non-zero only on cells a-1..a+1 of the parcel's cell a, the half-cell-shifted
// one on a-1..a+1 or a..a+2, and which of the two follows from |r| >= 1.5 at
// the ends (weights there are exactly +0).  So each parcel carries 3 x 27
// weights, each the same product (w1*w2)*w3 of the same 1-D values the
// reference forms; skipping the exact zeros leaves every sum unchanged.
//
// Spreading is deterministic: every (node, contribution) pair is emitted in
// part order, stably sorted by node, and each touched node sums its own run in
// that order -- the order in which the reference's serial loop over part(1:np)
// accumulates into fx.  Interpolation reads the halo layers directly, so the
// spread kernel refreshes the periodic mirrors of every node it updates.
#include <mutex>

#include "common.cuh"
#include "kernels.cuh"
#include "prims.cuh"

namespace ibmdem {

namespace {

// Correctly rounded x/3 with three FP64 operations (Markstein's correction
// step, P. Markstein, IBM J. Res. Dev. 34(1), 1990): q0 = x*RN(1/3) is within an
// ulp of x/3, r = x - 3*q0 is exact, and q0 + r*RN(1/3) is within 2^-50 ulp of
// x/3.  Since x/(3*ulp) always has fractional part 0, 1/3 or 2/3, x/3 is never
// nearer than ulp/6 to a rounding midpoint, so the final rounding is the
// correctly rounded quotient for every finite x (tests/test_gpu_division.py
// compares it with IEEE division).  x/6 = RN(x/3)*0.5 exactly (normal range).
__device__ inline double div3(double x) {
  const double c = 0x1.5555555555555p-2;  // RN(1/3)
  const double q0 = __dmul_rn(x, c);
  const double r = __fma_rn(-q0, 3.0, x);
  return __fma_rn(r, c, q0);
}

// x / dt, correctly rounded, without a division.  With 1/dt split as
// y + yl (y = RN(1/dt)), q0 = RN(x*y + RN(x*yl)) lies within half an ulp and a
// few 2^-105 of x/dt, so it is a faithful quotient and its remainder
// r = x - dt*q0 is exact in one FMA; RN(q0 + r*y) is then RN(x/dt) (Markstein's
// correction theorem; a plain RN(x*y) can miss x/dt by 1.5 ulp when 1/dt is
// rounded by a full half ulp, which is why div3's single product is not enough
// for an arbitrary dt).  The theorem needs r clear of the subnormal range and
// no overflow: x's exponent is checked with integer ops, and the division is
// taken outside 2^-723 <= |x| < 2^777 (and for x = 0).
__device__ inline double div_dt(double x, const Geom& g) {
  const int ex = (int)((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ff;
  if (!g.divDt || ex < 300 || ex > 1800) return x / g.dt;
  const double q0 = __fma_rn(x, g.rdt, __dmul_rn(x, g.rdtLo));
  const double r = __fma_rn(-q0, g.dt, x);
  return __fma_rn(r, g.rdt, q0);
}

// 0.0 + t and 0.0 - t under round-to-nearest, with integer ops in place of an
// FP64 add: t and -t, except that the sum of opposite zeros is +0.0
__device__ inline double zero_plus(double t) {
  const long long b = __double_as_longlong(t);
  return __longlong_as_double(b == (long long)0x8000000000000000ull ? 0ll : b);
}
__device__ inline double zero_minus(double t) {
  const long long b = __double_as_longlong(t);
  return __longlong_as_double(b == 0 ? 0ll : b ^ (long long)0x8000000000000000ull);
}

// one axis of DeltaFunction3D (interpolation.F90:7-30): the three points of a
// window.  Each point is the reference's expression for its distance r:
//   r <= 0.5:        (1 + sqrt(1 - 3 r r)) / 3
//   0.5 < r <= 1.5:  ((5 - 3 r - sqrt(1 - 3 (1 - r)(1 - r))) / 3) / 2
//   else             0
// The outer points of a window sit at u + 1/2 and u - 3/2 cells from the
// parcel (u its offset in the middle cell), so 1 - r is 1/2 - u and u - 1/2:
// when both differences are exact (Sterbenz, away from the origin) the two
// square roots have the same argument, bit for bit, and the second is not
// issued.  The arguments are compared, so the sharing never changes a bit.
// delta1 is one point.
template <int UNIT_H>
__device__ inline double delta1(double xcp, double h) {
  double r = fabs(UNIT_H ? xcp : xcp / h);
  if (r <= 0.5) return div3(1.0 + sqrt(1.0 - 3.0 * r * r));
  if (r <= 1.5) return div3(5.0 - 3.0 * r - sqrt(1.0 - 3.0 * ((1.0 - r) * (1.0 - r)))) * 0.5;
  return 0.0;
}
template <int UNIT_H>
__device__ inline void delta_triple(const double x[3], double h, double w[3]) {
  w[1] = delta1<UNIT_H>(x[1], h);
  const double r0 = fabs(UNIT_H ? x[0] : x[0] / h), r2 = fabs(UNIT_H ? x[2] : x[2] / h);
  if (r0 > 0.5 && r0 <= 1.5 && r2 > 0.5 && r2 <= 1.5) {
    // both outer points in the middle branch
    const double a0 = 1.0 - 3.0 * ((1.0 - r0) * (1.0 - r0));
    const double a2 = 1.0 - 3.0 * ((1.0 - r2) * (1.0 - r2));
    const double s0 = sqrt(a0);
    const double s2 = __double_as_longlong(a2) == __double_as_longlong(a0) ? s0 : sqrt(a2);
    w[0] = div3(5.0 - 3.0 * r0 - s0) * 0.5;
    w[2] = div3(5.0 - 3.0 * r2 - s2) * 0.5;
  } else {
    w[0] = delta1<UNIT_H>(x[0], h);
    w[2] = delta1<UNIT_H>(x[2], h);
  }
}

__device__ inline void window_start(const int4& wn, int comp, int& sx, int& sy, int& sz) {
  sx = wn.x - 1 + (comp == 0 ? (wn.w & 1) : 0);
  sy = wn.y - 1 + (comp == 1 ? ((wn.w >> 1) & 1) : 0);
  sz = wn.z - 1 + (comp == 2 ? ((wn.w >> 2) & 1) : 0);
}

// Mark the interior nodes of parcel window wn in the touched-node bits, all
// three components: bits ilo..ihi of each row the window covers, one atomic
// OR per row (and word).
__device__ inline void mark_window(const Geom& g, const int4& wn, unsigned* flags) {
  for (int comp = 0; comp < 3; ++comp) {
    int sx, sy, sz;
    window_start(wn, comp, sx, sy, sz);
    const int ilo = max(sx, 1), ihi = min(sx + 2, g.n[0]);
    if (ihi < ilo) continue;
    const unsigned run = (1u << (ihi - ilo + 1)) - 1u;
    for (int kz = 0; kz < 3; ++kz)
      for (int ky = 0; ky < 3; ++ky) {
        const int j = sy + ky, k = sz + kz;
        if (j < 1 || j > g.n[1] || k < 1 || k > g.n[2]) continue;
        const long long b0 = comp * g.nint + ((long long)(k - 1) * g.n[1] + (j - 1)) * g.n[0] + (ilo - 1);
        const int sh = (int)(b0 & 31);
        atomicOr(&flags[b0 >> 5], run << sh);
        if (sh + (ihi - ilo + 1) > 32) atomicOr(&flags[(b0 >> 5) + 1], run >> (32 - sh));
      }
  }
}

// mark the windows of all parcels, read in cell order so that a warp's ORs
// fall on neighbouring nodes (when the weights did not mark them)
__global__ void k_touch(Geom g, const Counters* cnt, const int4* winC, unsigned* flags) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= cnt->np) return;
  mark_window(g, winC[e], flags);
}

template <int UNIT_H>
__global__ void __launch_bounds__(kBlock) k_weights(Recs R, Geom g, Counters* cnt, int locals, double* W,
                                                    int4* win, int* cntInt, unsigned* touch) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int e = locals ? t : cnt->npLocal + t;
  if (locals ? (e >= cnt->npLocal) : (e >= cnt->np)) return;
  int a[3];
  cell_coords(g, R.I(I_CELL, e), a[0], a[1], a[2]);
  double wu[3][3], ws[3][3];
  int flags = 0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double xp = R.D(D_X + d, e), h = g.h[d];
    double dl[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      // xc = (i-0.5d0)*dx (initialization.F90:251); deltax = xp - xc (GetWeight)
      double xc = ((double)(a[d] - 1 + q) - 0.5);
      if (!UNIT_H) xc = xc * h;
      dl[q] = xp - xc;
    }
    delta_triple<UNIT_H>(dl, h, wu[d]);
    // half-cell shifted component: deltax + 0.5d0*di
    double s0 = dl[0] + g.halfh[d], s3 = dl[3] + g.halfh[d];
    double r0 = fabs(UNIT_H ? s0 : s0 / h), r3 = fabs(UNIT_H ? s3 : s3 / h);
    int st = r0 < 1.5 ? 0 : 1;
    if (r0 < 1.5 && r3 < 1.5) set_err(cnt, E_WINDOW, e);
    flags |= st << d;
    double xs[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) xs[q] = (st ? dl[q + 1] : dl[q]) + g.halfh[d];
    delta_triple<UNIT_H>(xs, h, ws[d]);
  }
  int total = 0;
  double4_32a* out = reinterpret_cast<double4_32a*>(W + (size_t)e * kWStride);
#pragma unroll
  for (int comp = 0; comp < 3; ++comp) {
    int cntAx[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      int s = a[d] - 1 + (d == comp ? ((flags >> d) & 1) : 0);
      int lo = max(s, 1), hi = min(s + 2, g.n[d]);
      cntAx[d] = hi >= lo ? hi - lo + 1 : 0;
    }
    total += cntAx[0] * cntAx[1] * cntAx[2];
    double wc[28];
#pragma unroll
    for (int ky = 0; ky < 3; ++ky)
#pragma unroll
      for (int kx = 0; kx < 3; ++kx) {
        double w1 = comp == 0 ? ws[0][kx] : wu[0][kx];
        double w2 = comp == 1 ? ws[1][ky] : wu[1][ky];
        double w12 = w1 * w2;
#pragma unroll
        for (int kz = 0; kz < 3; ++kz) {
          double w3 = comp == 2 ? ws[2][kz] : wu[2][kz];
          double wt = w12 * w3;
          if (!UNIT_H) wt = wt / g.hprod;
          wc[kz * 9 + ky * 3 + kx] = wt;
        }
      }
    wc[27] = 0.0;
#pragma unroll
    for (int q = 0; q < 7; ++q) out[comp * 7 + q] = make_double4_32a(wc[4 * q], wc[4 * q + 1], wc[4 * q + 2], wc[4 * q + 3]);
  }
  const int4 wn = make_int4(a[0], a[1], a[2], flags);
  win[e] = wn;
  cntInt[e] = total;
  // the touched-node bits of the spread plan, set here where the windows are
  // made (the atomics go out beside the FP64 work)
  mark_window(g, wn, touch);
}


// ---- spread plan -------------------------------------------------------------
// A node (component c, interior (i,j,k)) receives from every parcel whose
// c-window covers it.  Windows start at cell-1 on the unshifted axes and at
// cell-1 or cell on the shifted axis, so the candidates live in a 4x3x3 block
// of cells (4 along axis c).  Each plan entry keeps the contributing root
// parcel (images share their source's fdrag*vol) and its weight, so spreading
// streams the plan sequentially.


// compaction of the flag bits into the sorted node-key list (128 flags per thread)
__global__ void k_flag_count(const uint4* flags, long long nvec, int* blockCnt) {
  __shared__ int sh[kBlock / 32];
  long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int c = 0;
  if (v < nvec) {
    uint4 q = flags[v];
    c = __popc(q.x) + __popc(q.y) + __popc(q.z) + __popc(q.w);
  }
  for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < kBlock / 32; ++w) t += sh[w];
    blockCnt[blockIdx.x] = t;
  }
}
__global__ void k_flag_emit(const uint4* flags, long long nvec, long long nflags, const int* blockOff,
                            uint32_t* keys, long long capRuns, Counters* cnt, long long nint) {
  __shared__ int sh[kBlock / 32];
  long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t w4[4] = {0, 0, 0, 0};
  if (v < nvec) {
    uint4 q = flags[v];
    w4[0] = q.x; w4[1] = q.y; w4[2] = q.z; w4[3] = q.w;
  }
  int c = __popc(w4[0]) + __popc(w4[1]) + __popc(w4[2]) + __popc(w4[3]);
  // exclusive prefix of c over the block
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = c;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[warp] = x;
  __syncthreads();
  int base = blockOff[blockIdx.x];
  for (int w = 0; w < warp; ++w) base += sh[w];
  int pos = base + x - c;
  const long long f0 = v * 128;
  // the first run of velocity components 1 and 2: the flags set below their
  // first node, counted by the thread whose 128 flags hold that node
#pragma unroll
  for (int comp = 1; comp < 3; ++comp) {
    const long long first = comp * nint;
    if (first >= f0 && first < f0 + 128) {
      const int b = (int)(first - f0);
      int below = 0;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int nb = min(max(b - 32 * q, 0), 32);
        below += __popc(nb == 32 ? w4[q] : (w4[q] & ((1u << nb) - 1u)));
      }
      cnt->compStart[comp] = min(pos + below, cnt->nRuns);
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    uint32_t w = w4[q];
    while (w) {
      const long long f = f0 + 32 * q + (__ffs(w) - 1);
      w &= w - 1u;
      if (f < nflags) {
        if (pos < capRuns) keys[pos] = (uint32_t)f;
        ++pos;
      }
    }
  }
}

// touched nodes beyond the run capacity are dropped and reported
__global__ void k_set_runs(Counters* cnt, const int* total, long long capRuns) {
  const int t = *total;
  if (t > capRuns) set_err(cnt, E_PLANCAP, t);
  cnt->compStart[0] = 0;
  cnt->compStart[3] = (int)min((long long)t, capRuns);
  cnt->nRuns = (int)min((long long)t, capRuns);
}

// The fill works on sub-groups: up to kSubMax consecutive touched nodes of one
// grid row (same component, j and k), taken from a warp's 32 runs.  The warp
// gathers the parcels of the row's candidate cells once, keeps those whose
// window covers the row in y and z and reaches the sub-group in x, and sorts
// them by part index.  A kept parcel covers the three nodes sx..sx+2 of the
// row, so each node's contributors in part order are the sorted list filtered
// by sx in [i-2, i]: one ballot per node, whose mask stays in the node's lane,
// and each kept parcel writes its own entries from those masks.  The entries
// (parcel << 7 | slot) are staged per warp in shared memory; the block
// reserves its contribution range with one atomic (the 256 runs of a block own
// one contiguous range in run order, which the spread relies on) and writes
// (root | comp << 30, weight) with consecutive lanes on consecutive entries.  A
// sub-group with more than kLCap kept parcels is halved until it fits; a
// single node with more than kLCap contributors, or a warp whose entries exceed
// its staging, is written straight into the plan range after the reservation.
__device__ inline void node_coords(const Geom& g, uint32_t key, int& comp, int& i, int& j, int& k) {
  const uint32_t c = g.fdNint.div(key);
  const uint32_t node = key - c * (uint32_t)g.nint;
  const uint32_t row = g.fdN0.div(node);
  const uint32_t kk = g.fdN1.div(row);
  comp = (int)c;
  i = (int)(node - row * (uint32_t)g.n[0]) + 1;
  j = (int)(row - kk * (uint32_t)g.n[1]) + 1;
  k = (int)kk + 1;
}

constexpr int kSubMax = 16;     // nodes per sub-group (a power of two: the node scan)
constexpr int kLCap = 64;       // kept parcels per sub-group (two per lane)
constexpr int kStageCap = 512;  // staged entries per warp
constexpr int kPlanWarps = kBlock / 32;
constexpr unsigned kFull = 0xffffffffu;

// Gather the parcels of the candidate cells of nodes iFirst..iLast of row
// (comp, j, k) whose window covers the row and reaches [iFirst, iLast]; the
// first kLCap go to key (part index) and aux (sx - iFirst + 2 | (dz*3+dy) << 8).
// Returns how many there are (all lanes).
__device__ inline int gather_row(const Geom& g, int comp, int iFirst, int iLast, int j, int k,
                                 const int* __restrict__ cellStart, const int* __restrict__ cellItems,
                                 const int4* __restrict__ winC, uint32_t* key, uint32_t* aux, int lane) {
  const int xlo = iFirst - (comp == 0 ? 2 : 1), xhi = iLast + 1;
  const int ylo = j - (comp == 1 ? 2 : 1), zlo = k - (comp == 2 ? 2 : 1);
  const int ny = comp == 1 ? 4 : 3, nr = ny * (comp == 2 ? 4 : 3);  // candidate cell rows (<= 12)
  int q0 = 0, len = 0;
  if (lane < nr) {
    // lane / ny for ny = 3 or 4 and lane < 16: (lane * 11) >> 5 is lane / 3 there
    const int dz = ny == 4 ? lane >> 2 : (lane * 11) >> 5;
    const int cy = ylo + (lane - dz * ny), cz = zlo + dz;
    // cell_id(g, xlo, cy, cz) - 1 in 32 bits (the cell count fits an int)
    const int c0 = ((cz + 1) * g.nj + (cy + 1)) * g.ni + (xlo + 1);
    q0 = cellStart[c0];
    len = cellStart[c0 + 1 + (xhi - xlo)] - q0;
  }
  int inc = len;  // inclusive prefix over lanes 0..15 (rows past nr are empty)
#pragma unroll
  for (int o = 1; o < 16; o <<= 1) {
    const int y = __shfl_up_sync(kFull, inc, o);
    if (lane >= o) inc += y;
  }
  const int excl = inc - len;
  const int total = __shfl_sync(kFull, inc, 15);
  const unsigned lt = (1u << lane) - 1u;
  int m = 0;
  for (int f0 = 0; f0 < total; f0 += 32) {
    const int f = f0 + lane;
    // the last row whose first candidate is at or before f
    int row = 0;
#pragma unroll
    for (int step = 8; step; step >>= 1) {
      const int probe = __shfl_sync(kFull, excl, row + step);
      if (probe <= f) row += step;
    }
    const int rq = __shfl_sync(kFull, q0, row);
    const int rx = __shfl_sync(kFull, excl, row);
    bool keep = false;
    uint32_t pk = 0, pa = 0;
    if (f < total) {
      const int q = rq + (f - rx);
      int sx, sy, sz;
      window_start(winC[q], comp, sx, sy, sz);
      const int dy = j - sy, dz = k - sz;
      keep = (unsigned)dy <= 2u && (unsigned)dz <= 2u && sx <= iLast && sx + 2 >= iFirst;
      if (keep) {
        pk = (uint32_t)cellItems[q];
        pa = (uint32_t)(sx - iFirst + 2) | (uint32_t)(dz * 3 + dy) << 8;
      }
    }
    const unsigned mk = __ballot_sync(kFull, keep);
    if (keep) {
      const int at = m + __popc(mk & lt);
      if (at < kLCap) {
        key[at] = pk;
        aux[at] = pa;
      }
    }
    m += __popc(mk);
  }
  return m;
}

// Contributors of one node straight into out[0..), part order (a node with more
// than kLCap of them; one lane).  Returns how many.
__device__ inline int scan_node_into(const Geom& g, int comp, int i, int j, int k, const int* __restrict__ cellStart,
                                     const int* __restrict__ cellItems, const int4* __restrict__ winC,
                                     uint32_t* out) {
  const int alo = i - (comp == 0 ? 2 : 1), ahi = i + 1;
  const int blo = j - (comp == 1 ? 2 : 1), bhi = j + 1;
  const int clo = k - (comp == 2 ? 2 : 1), chi = k + 1;
  int t = 0;
  for (int cz = clo; cz <= chi; ++cz)
    for (int cy = blo; cy <= bhi; ++cy) {
      const int c0 = cell_id(g, alo, cy, cz);
      const int q0 = cellStart[c0 - 1], q1 = cellStart[c0 + (ahi - alo)];
      for (int q = q0; q < q1; ++q) {
        int sx, sy, sz;
        window_start(winC[q], comp, sx, sy, sz);
        const int dx = i - sx, dy = j - sy, dz = k - sz;
        if ((unsigned)dx > 2u || (unsigned)dy > 2u || (unsigned)dz > 2u) continue;
        out[t++] = ((uint32_t)cellItems[q] << 7) | (uint32_t)(comp * 27 + dz * 9 + dy * 3 + dx);
      }
    }
  for (int a = 1; a < t; ++a) {
    const uint32_t v = out[a];
    int at = a;
    while (at > 0 && out[at - 1] > v) {
      out[at] = out[at - 1];
      --at;
    }
    out[at] = v;
  }
  return t;
}

// The warp's sub-groups in lane order: entries (parcel << 7 | slot) to
// out[pos] for pos < outCap, each lane's node count and offset.  With direct
// set, out is the warp's plan range and oversized nodes are scanned into it;
// otherwise they only count (*needDirect is set).  Returns the warp's total.
__device__ inline int fill_subgroups(const Geom& g, unsigned starts, int nValid, int comp, int i, int j, int k,
                                     const int* __restrict__ cellStart, const int* __restrict__ cellItems,
                                     const int4* __restrict__ winC, uint32_t* key, uint32_t* aux, uint32_t* out,
                                     int outCap, bool direct, int lane, int& myCnt, int& myOff, bool& needDirect) {
  const unsigned lt = (1u << lane) - 1u;
  int off = 0;
  unsigned rest = starts;
  while (rest) {
    const int l0 = __ffs(rest) - 1;
    rest &= rest - 1u;
    int l1 = (rest ? __ffs(rest) - 1 : nValid) - 1;
    const int sc = __shfl_sync(kFull, comp, l0);
    const int sj = __shfl_sync(kFull, j, l0), sk = __shfl_sync(kFull, k, l0);
    const int iFirst = __shfl_sync(kFull, i, l0);
    int m = gather_row(g, sc, iFirst, __shfl_sync(kFull, i, l1), sj, sk, cellStart, cellItems, winC, key, aux, lane);
    while (m > kLCap && l1 > l0) {
      // too many for one list: the first half now, the second as a sub-group of its own
      const int mid = l0 + ((l1 - l0 + 1) >> 1);
      rest |= 1u << mid;
      l1 = mid - 1;
      m = gather_row(g, sc, iFirst, __shfl_sync(kFull, i, l1), sj, sk, cellStart, cellItems, winC, key, aux, lane);
    }
    if (m > kLCap) {
      // one node with more than kLCap contributors (m counts exactly them)
      if (direct && lane == l0) scan_node_into(g, sc, iFirst, sj, sk, cellStart, cellItems, winC, out + off);
      if (lane == l0) {
        myCnt = m;
        myOff = off;
      }
      needDirect = true;
      off += m;
      __syncwarp();
      continue;
    }
    __syncwarp();
    // part order: rank of each kept parcel among the others (part indices are distinct)
    uint32_t ek[2], ea[2];
    int rk[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int e = lane + 32 * u;
      ek[u] = e < m ? key[e] : 0xffffffffu;
      ea[u] = e < m ? aux[e] : 0u;
      rk[u] = 0;
    }
    if (m <= 32) {
#pragma unroll 4
      for (int f = 0; f < m; ++f) rk[0] += __shfl_sync(kFull, ek[0], f) < ek[0];
    } else {
      for (int f = 0; f < m; ++f) {
        const uint32_t kf = key[f];
        rk[0] += kf < ek[0];
        rk[1] += kf < ek[1];
      }
    }
    __syncwarp();
#pragma unroll
    for (int u = 0; u < 2; ++u)
      if (lane + 32 * u < m) {
        key[rk[u]] = ek[u];
        aux[rk[u]] = ea[u];
      }
    __syncwarp();
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int e = lane + 32 * u;
      ek[u] = e < m ? key[e] : 0u;
      ea[u] = e < m ? aux[e] : 0u;
    }
    __syncwarp();
    // The sub-group's nodes are iFirst + t, t < nn <= kSubMax.  One ballot per
    // node (and slot) leaves node t's contributor masks in lane t; a scan over
    // those lanes gives each node's offset, and each kept parcel then writes
    // its own (up to three) entries at the node's offset plus its rank among
    // the node's contributors (slots, then lanes, are in part order).
    const int nn = l1 - l0 + 1;
    unsigned mask0 = 0u, mask1 = 0u;
    const int sxr0 = (int)(ea[0] & 0xffu) - 2;  // sx - iFirst
    if (m <= 32) {
      for (int t = 0; t < nn; ++t) {
        const unsigned b0 = __ballot_sync(kFull, lane < m && (unsigned)(t - sxr0) <= 2u);
        if (lane == t) mask0 = b0;
      }
    } else {
      const int sxr1 = (int)(ea[1] & 0xffu) - 2;
      for (int t = 0; t < nn; ++t) {
        const unsigned b0 = __ballot_sync(kFull, (unsigned)(t - sxr0) <= 2u);
        const unsigned b1 = __ballot_sync(kFull, lane + 32 < m && (unsigned)(t - sxr1) <= 2u);
        if (lane == t) {
          mask0 = b0;
          mask1 = b1;
        }
      }
    }
    const int cntT = __popc(mask0) + __popc(mask1);
    int incl = cntT;
#pragma unroll
    for (int o = 1; o < kSubMax; o <<= 1) {
      const int y = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += y;
    }
    const int exclT = incl - cntT;
    const int subTotal = __shfl_sync(kFull, incl, kSubMax - 1);
    {
      const uint32_t entry = (ek[0] << 7) | (uint32_t)(sc * 27 + 3 * (int)(ea[0] >> 8));
#pragma unroll
      for (int dx = 0; dx < 3; ++dx) {
        const int t = sxr0 + dx;
        const int tc = min(max(t, 0), kSubMax - 1);
        const unsigned M0 = __shfl_sync(kFull, mask0, tc);
        const int O = __shfl_sync(kFull, exclT, tc);
        if (lane < m && t >= 0 && t < nn) {
          const int at = off + O + __popc(M0 & lt);
          if (at < outCap) out[at] = entry + (uint32_t)dx;
        }
      }
    }
    if (m > 32) {
      const int sxr1 = (int)(ea[1] & 0xffu) - 2;
      const uint32_t entry = (ek[1] << 7) | (uint32_t)(sc * 27 + 3 * (int)(ea[1] >> 8));
#pragma unroll
      for (int dx = 0; dx < 3; ++dx) {
        const int t = sxr1 + dx;
        const int tc = min(max(t, 0), kSubMax - 1);
        const unsigned M0 = __shfl_sync(kFull, mask0, tc), M1 = __shfl_sync(kFull, mask1, tc);
        const int O = __shfl_sync(kFull, exclT, tc);
        if (lane + 32 < m && t >= 0 && t < nn) {
          const int at = off + O + __popc(M0) + __popc(M1 & lt);
          if (at < outCap) out[at] = entry + (uint32_t)dx;
        }
      }
    }
    const int src = min(max(lane - l0, 0), kSubMax - 1);
    const int cN = __shfl_sync(kFull, cntT, src), oN = __shfl_sync(kFull, exclT, src);
    if (lane >= l0 && lane <= l1) {
      myCnt = cN;
      myOff = off + oN;
    }
    off += subTotal;
  }
  return off;
}

__global__ void __launch_bounds__(kBlock, 6) k_plan_fill(Geom g, Counters* cnt, const uint32_t* __restrict__ runKey,
                                                         const int* __restrict__ cellStart,
                                                         const int* __restrict__ cellItems,
                                                         const int4* __restrict__ winC,
                                                         const double* __restrict__ W,
                                                         const int* __restrict__ imgSrc, int* runStart, int* runCnt,
                                                         uint32_t* planRoot, double* planW,
                                                         unsigned long long* cursor, long long capContrib) {
  __shared__ int warpSum[kPlanWarps];
  __shared__ long long blockBase;
  __shared__ uint32_t sKey[kPlanWarps][kLCap], sAux[kPlanWarps][kLCap];
  __shared__ uint32_t sStage[kPlanWarps][kStageCap];
  const long long nRuns = cnt->nRuns;
  const int npLocal = cnt->npLocal;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t* key = sKey[warp];
  uint32_t* aux = sAux[warp];
  uint32_t* stage = sStage[warp];
  for (long long r0 = (long long)blockIdx.x * kBlock; r0 < nRuns; r0 += (long long)gridDim.x * kBlock) {
    const long long r = r0 + threadIdx.x;
    const bool has = r < nRuns;
    const uint32_t rkey = has ? runKey[r] : 0u;
    int comp = 0, i = 1, j = 1, k = 1;
    if (has) node_coords(g, rkey, comp, i, j, k);
    // sub-groups: consecutive nodes of one row, split every kSubMax nodes
    const uint32_t rowKey = rkey - (uint32_t)(i - 1);
    const uint32_t prevRow = __shfl_up_sync(kFull, rowKey, 1);
    const int prevI = __shfl_up_sync(kFull, i, 1);
    const unsigned valid = __ballot_sync(kFull, has);  // lanes 0..nValid-1
    const int nValid = __popc(valid);
    bool start = lane == 0 || rowKey != prevRow || i != prevI + 1;
    unsigned starts = __ballot_sync(kFull, start && has);
    const unsigned upTo = lane == 31 ? kFull : (2u << lane) - 1u;
    const int lastStart = 31 - __clz(starts & upTo);
    start = start || (lane - lastStart) % kSubMax == 0;
    starts = __ballot_sync(kFull, start && has);

    int myCnt = 0, myOff = 0;
    bool needDirect = false;
    const int total = fill_subgroups(g, starts, nValid, comp, i, j, k, cellStart, cellItems, winC, key, aux, stage,
                                     kStageCap, false, lane, myCnt, myOff, needDirect);
    if (total > kStageCap) needDirect = true;
    // one reservation for the block, warps in run order
    if (lane == 0) warpSum[warp] = total;
    __syncthreads();
    long long pre = 0, tot = 0;
#pragma unroll
    for (int w = 0; w < kPlanWarps; ++w) {
      pre += w < warp ? warpSum[w] : 0;
      tot += warpSum[w];
    }
    if (threadIdx.x == 0) blockBase = (long long)atomicAdd(cursor, (unsigned long long)tot);
    __syncthreads();
    const long long o = blockBase + pre;
    if (has) {
      runStart[r] = (int)(o + myOff);
      runCnt[r] = myCnt;
    }
    if (o + total > capContrib) {
      if (lane == 0 && total > 0) set_err(cnt, E_PLANCAP, (int)(r0 + 32 * warp));
    } else {
      if (needDirect) {
        // again, with the entries written straight into the warp's range
        int c2 = 0, o2 = 0;
        bool nd = false;
        fill_subgroups(g, starts, nValid, comp, i, j, k, cellStart, cellItems, winC, key, aux, planRoot + o,
                       total, true, lane, c2, o2, nd);
        __syncwarp();
      }
      for (int t = lane; t < total; t += 32) {
        const uint32_t v = needDirect ? planRoot[o + t] : stage[t];
        const int p = (int)(v >> 7);
        const int slot = (int)(v & 127u);
        const int sc = slot / 27;
        const uint32_t root = (uint32_t)(p < npLocal ? p : imgSrc[p - npLocal]);
        planRoot[o + t] = root | ((uint32_t)sc << 30);
        planW[o + t] = W[(size_t)p * kWStride + sc * 28 + (slot - sc * 27)];
      }
    }
    __syncthreads();
  }
}

// windows of the cell items, in cell order
__global__ void k_win_by_cell(const Counters* cnt, const int* __restrict__ cellItems, const int4* __restrict__ win,
                              int4* winC) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < cnt->np) winC[q] = win[cellItems[q]];
}

__global__ void k_plan_total(Counters* cnt, const unsigned long long* cursor) {
  cnt->nContrib = (int)*cursor;
}


// Write the new value of interior node (i,j,k) of component comp where the
// fluid solver's halo refill puts it (FillGhostRegionForFluid,
// boundary.F90:122-147): per axis the node itself and, within the 2-cell halo
// of a face, its copy beyond the opposite face (periodic) or its mirror beyond
// that face with the sign flipped (solid wall, DealWithBoundaryFluid,
// boundary.F90:211-245).  Boundary() (fluid.F90:240-249) then zeroes the
// wall-normal component on the wall face and beyond it.
template <bool WALLS>
__device__ inline void put_mirrored(double* F, const Geom& g, int comp, int i, int j, int k, double val) {
  if (!WALLS) {
    int ox[2] = {0, 0}, oy[2] = {0, 0}, oz[2] = {0, 0};
    int nxo = 1, nyo = 1, nzo = 1;
    if (i <= kHalo) ox[nxo++] = g.n[0];
    else if (i > g.n[0] - kHalo) ox[nxo++] = -g.n[0];
    if (j <= kHalo) oy[nyo++] = g.n[1];
    else if (j > g.n[1] - kHalo) oy[nyo++] = -g.n[1];
    if (k <= kHalo) oz[nzo++] = g.n[2];
    else if (k > g.n[2] - kHalo) oz[nzo++] = -g.n[2];
    for (int c = 0; c < nzo; ++c)
      for (int b = 0; b < nyo; ++b)
        for (int a = 0; a < nxo; ++a) F[field_off(g, i + ox[a], j + oy[b], k + oz[c])] = val;
    return;
  }
  int pos[3][2], neg[3][2], cnt[3];
  const int id[3] = {i, j, k};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    pos[d][0] = id[d];
    neg[d][0] = 0;
    cnt[d] = 1;
    const int n = g.n[d];
    if (id[d] <= kHalo) {
      pos[d][1] = g.wall[d] ? 1 - id[d] : id[d] + n;
      neg[d][1] = g.wall[d];
      cnt[d] = 2;
    } else if (id[d] > n - kHalo) {
      pos[d][1] = g.wall[d] ? 2 * n + 1 - id[d] : id[d] - n;
      neg[d][1] = g.wall[d];
      cnt[d] = 2;
    }
  }
  const int nc = g.n[comp];
  for (int c = 0; c < cnt[2]; ++c)
    for (int b = 0; b < cnt[1]; ++b)
      for (int a = 0; a < cnt[0]; ++a) {
        const int p[3] = {pos[0][a], pos[1][b], pos[2][c]};
        double v = (neg[0][a] ^ neg[1][b] ^ neg[2][c]) ? -val : val;
        if (g.wall[comp] && (p[comp] <= 1 || p[comp] >= nc + 1)) v = 0.0;
        F[field_off(g, p[0], p[1], p[2])] = v;
      }
}

struct Fields {
  double *u, *v, *w, *u0, *v0, *w0, *fx, *fy, *fz;
  __device__ double* U(int c) const { return c == 0 ? u : (c == 1 ? v : w); }
  __device__ double* U0(int c) const { return c == 0 ? u0 : (c == 1 ? v0 : w0); }
  __device__ double* F(int c) const { return c == 0 ? fx : (c == 1 ? fy : fz); }
};

// start of FirstOrderForwardEuler's particle side (fluid.F90:255-263): fdrag=0,
// fx=fy=fz=0; with `frozen`, also restore the fluid where the last spread
// changed it.
template <bool WALLS>
__global__ void k_mdf_reset(Recs R, Geom g, Counters* cnt, Fields fl, const uint32_t* lastNodes, double* fCur,
                            int frozen) {
  const long long nLast = cnt->nLast, nRuns = cnt->nRuns, nl = cnt->npLocal;
  const long long n = max(nLast, max(nRuns, nl));
  GRID_STRIDE(t, n) {
    if (t < nLast) {
      int comp, i, j, k;
      node_coords(g, lastNodes[t], comp, i, j, k);
      long long off = field_off(g, i, j, k);
      fl.F(comp)[off] = 0.0;
      if (frozen) put_mirrored<WALLS>(fl.U(comp), g, comp, i, j, k, fl.U0(comp)[off]);
    }
    if (t < nRuns) fCur[t] = 0.0;
    if (t < nl) {
      R.D(D_FDRAG, (int)t) = 0.0;
      R.D(D_FDRAG + 1, (int)t) = 0.0;
      R.D(D_FDRAG + 2, (int)t) = 0.0;
    }
  }
}

// The reset of FirstOrderForwardEuler's particle side (fluid.F90:255-263:
// fdrag = 0, fx = fy = fz = 0, and in a frozen-fluid step the field restored)
// when the forcing loop runs: the first iteration's kernels take fdrag and
// fxOld as 0 and the frozen field as the old velocity, and every node the new
// plan touches is rewritten by the first spread, so only the nodes the last
// spread wrote and the new plan does not touch (the touched-node bits) are
// reset here.
template <bool WALLS>
__global__ void k_mdf_stale(Geom g, const Counters* cnt, Fields fl, const uint32_t* __restrict__ lastNodes,
                            const unsigned* __restrict__ touch, int frozen) {
  const long long nLast = cnt->nLast;
  GRID_STRIDE(t, nLast) {
    const uint32_t key = lastNodes[t];
    if ((touch[key >> 5] >> (key & 31u)) & 1u) continue;
    int comp, i, j, k;
    node_coords(g, key, comp, i, j, k);
    const long long off = field_off(g, i, j, k);
    fl.F(comp)[off] = 0.0;
    if (frozen) put_mirrored<WALLS>(fl.U(comp), g, comp, i, j, k, fl.U0(comp)[off]);
  }
}

// UpdateFluidVelocityOnLagrangianPoints (ZJS_VOLUMEFRACTION_DEM.F90:2-36);
// blockIdx.y is the velocity component.  first: bit 0, the forcing loop's first iteration (fdrag was just reset to 0);
// bit 1, the field is read from the frozen copy (the first iteration of a
// frozen-fluid step, before any spread of this step wrote the working field).
template <int UNIT_H>
__device__ __forceinline__ void interp_one(const Recs& R, const Geom& g, const double* __restrict__ W,
                                           const int4* __restrict__ win, const Fields& fl, double* fv, int comp,
                                           int first, int m) {
  const int cap = R.cap;
  const double* __restrict__ F = (first & 2) ? fl.U0(comp) : fl.U(comp);
  int sx, sy, sz;
  window_start(win[m], comp, sx, sy, sz);
  const double4_32a* Wc = reinterpret_cast<const double4_32a*>(W + (size_t)m * kWStride + comp * 28);
  double wv[28];
#pragma unroll
  for (int q = 0; q < 7; ++q) {
    double4_32a t4 = Wc[q];
    wv[4 * q] = t4.x;
    wv[4 * q + 1] = t4.y;
    wv[4 * q + 2] = t4.z;
    wv[4 * q + 3] = t4.w;
  }
  double ulp = 0.0;
#pragma unroll
  for (int kz = 0; kz < 3; ++kz)
#pragma unroll
    for (int ky = 0; ky < 3; ++ky) {
      const double* row = F + field_off(g, sx, sy + ky, sz + kz);
#pragma unroll
      for (int kx = 0; kx < 3; ++kx) {
        double t = wv[kz * 9 + ky * 3 + kx] * row[kx];
        if (!UNIT_H) {
          t = t * g.h[0];
          t = t * g.h[1];
          t = t * g.h[2];
        }
        ulp = (kz | ky | kx) ? ulp + t : zero_plus(t);  // 0.0 + t first
      }
    }
  const double vp = R.D(D_V + comp, m);
  R.D(D_VGAP + comp, m) = ulp - vp;
  // relaxfactor * (ulp - vp) / dt with relaxfactor = 1: the product is exact;
  // after the reset fdrag = 0, so 0.0 + q is q (+0 for a -0)
  const double q = div_dt(ulp - vp, g);
  const double fd = (first & 1) ? zero_plus(q) : R.D(D_FDRAG + comp, m) + q;
  R.D(D_FDRAG + comp, m) = fd;
  fv[(size_t)comp * cap + m] = fd * R.D(D_VOL, m);
}

template <int UNIT_H>
__global__ void __launch_bounds__(kBlock) k_interp(Recs R, Geom g, const Counters* cnt, const double* __restrict__ W,
                                                   const int4* __restrict__ win, Fields fl, double* fv, int comp0,
                                                   int first) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= cnt->npLocal) return;
  interp_one<UNIT_H>(R, g, W, win, fl, fv, comp0 + blockIdx.y, first, m);
}

// UpdateMomentumSourceTerm (ZJS_VOLUMEFRACTION_DEM.F90:38-67) per touched node;
// MODE 0: fused with VelocityPostGuess + halo refill, 1: spread only.
// 2560 staged products per block (20 KB) let 8 blocks share an SM (32 registers,
// under 24 KB of shared memory each, so that the SM keeps the 196 KB shared
// memory split and 60 KB of L1, which the kernels that run beside it in a batch
// of cases rely on); a block whose range holds more (markers far denser than the
// usual spacing) folds from global memory instead.
constexpr int kSpreadBlock = kBlock;  // touched nodes (threads) per spread block: one plan-fill block
constexpr int kSpreadBuf = 10 * kSpreadBlock;  // products per block held in shared memory
constexpr int kStageDepth = 4;    // plan loads in flight per thread while staging
constexpr int kLenBins = 64;
// A block takes 256 consecutive touched nodes (one contiguous plan range).
// Their products (fdrag*vol)*weight are formed in parallel from coalesced
// reads; a counting sort by run length then hands nodes of similar length to
// the same warp, so the FP64 lanes fold in step.  Each thread folds its node in
// part order -- the reference's fx = fx - fdrag*vol*weight, term by term --
// then applies the post-guess update with the periodic mirrors (MODE 0) or
// keeps fx and fxOld for a separate VelocityPostGuess (MODE 1).  (Folding the
// shortest and the longest node in one thread idles fewer FP64 lanes but
// leaves half the warps without work in the fold, and measured slower.)
// The chunks of 256 runs of block `blk` among `nBlk` blocks; the shared-memory
// buffers come from the kernel (prod: kSpreadBuf doubles, bins, order and
// sStart as in k_spread).
template <int MODE, bool WALLS, int FIRST>
__device__ __forceinline__ void spread_chunks(const Geom& g, const Counters* cnt, const int* __restrict__ runStart,
                                              const int* __restrict__ runCnt, const uint32_t* __restrict__ runKey,
                                              const uint32_t* __restrict__ planRoot,
                                              const double* __restrict__ planW, const double* __restrict__ fv,
                                              int cap, const Fields& fl, double* fCur, double* fPrev, int onlyComp,
                                              int blk, int nBlk, double* prod, int* bins, int* order, int* sStart) {
  const int nRuns = cnt->nRuns;  // run counts are ints (Counters)
  // one component's runs [rs, re) (onlyComp >= 0) or all of them; a block
  // always stages its whole 256-run range (contiguous in the plan) but writes
  // only its own component's nodes
  const int rs = onlyComp < 0 ? 0 : cnt->compStart[onlyComp];
  const int re = onlyComp < 0 ? nRuns : cnt->compStart[onlyComp + 1];
  for (int r0 = (rs / kSpreadBlock + blk) * kSpreadBlock; r0 < re; r0 += nBlk * kSpreadBlock) {
    const int nHere = min(kSpreadBlock, nRuns - r0);
    // this thread's own node: everything its epilogue needs, loaded up front
    const int myR = r0 + threadIdx.x;
    const bool has = (int)threadIdx.x < nHere;
    const bool mine = has && myR >= rs && myR < re;
    int comp = 0, i = 1, j = 1, k = 1, myLen = 0;
    long long off = 0;
    double uOld = 0.0, fo = 0.0;
    if (has) {
      node_coords(g, runKey[myR], comp, i, j, k);
      off = field_off(g, i, j, k);
      myLen = runCnt[myR];
      const int st = runStart[myR];
      sStart[threadIdx.x] = st;
      if ((int)threadIdx.x == nHere - 1) sStart[nHere] = st + myLen;
      // the first iteration: fxOld = 0 (the reset), and in a frozen-fluid step
      // the node's velocity is the frozen one
      fo = (FIRST & 1) ? 0.0 : fCur[myR];
      if (MODE == 0) uOld = (FIRST & 2) ? fl.U0(comp)[off] : fl.U(comp)[off];
    }
    if (threadIdx.x < kLenBins) bins[threadIdx.x] = 0;
    __syncthreads();
    const int base = sStart[0];
    const int total = sStart[nHere] - base;
    const bool staged = total <= kSpreadBuf;
    if (staged)
      for (int q0 = threadIdx.x; q0 < total; q0 += kStageDepth * kSpreadBlock) {
        // kStageDepth independent plan loads and gathers in flight per thread
        uint32_t rc[kStageDepth];
        double w[kStageDepth], a[kStageDepth];
#pragma unroll
        for (int u = 0; u < kStageDepth; ++u) {
          const int q = q0 + u * kSpreadBlock;
          rc[u] = q < total ? planRoot[base + q] : 0u;
          w[u] = q < total ? planW[base + q] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < kStageDepth; ++u)
          a[u] = q0 + u * kSpreadBlock < total ? fv[(size_t)(rc[u] >> 30) * cap + (rc[u] & 0x3fffffffu)] : 0.0;
#pragma unroll
        for (int u = 0; u < kStageDepth; ++u)
          if (q0 + u * kSpreadBlock < total) prod[q0 + u * kSpreadBlock] = a[u] * w[u];
      }
    const int bin = min(myLen, kLenBins - 1);
    if (has) atomicAdd(&bins[bin], 1);
    __syncthreads();
    if (threadIdx.x < 32) {  // exclusive prefix of the 64 bins by one warp
      int a0 = bins[threadIdx.x], a1 = bins[threadIdx.x + 32];
      int x0 = a0, x1 = a1;
      for (int o = 1; o < 32; o <<= 1) {
        int y0 = __shfl_up_sync(0xffffffffu, x0, o), y1 = __shfl_up_sync(0xffffffffu, x1, o);
        if (threadIdx.x >= o) {
          x0 += y0;
          x1 += y1;
        }
      }
      int t0 = __shfl_sync(0xffffffffu, x0, 31);
      bins[threadIdx.x] = x0 - a0;
      bins[threadIdx.x + 32] = t0 + x1 - a1;
    }
    __syncthreads();
    if (has) order[atomicAdd(&bins[bin], 1)] = threadIdx.x;
    __syncthreads();
    // fold a node of similar length to the warp's other nodes, in part order
    if ((int)threadIdx.x < nHere) {
      const int loc = order[threadIdx.x];
      const int s0 = sStart[loc] - base, n = sStart[loc + 1] - sStart[loc];
      // f = 0.0 - p1 - p2 - ..., the first subtraction exact without the FP64 pipe
      double f = 0.0;
      if (staged) {
        if (n > 0) {
          f = zero_minus(prod[s0]);
          for (int q = s0 + 1; q < s0 + n; ++q) f = f - prod[q];
          prod[s0] = f;
        }
      } else {
        for (int q = base + s0; q < base + s0 + n; ++q) {
          const uint32_t rc = planRoot[q];
          const double p = fv[(size_t)(rc >> 30) * cap + (rc & 0x3fffffffu)] * planW[q];
          f = q == base + s0 ? zero_minus(p) : f - p;
        }
        prod[loc] = f;
      }
    }
    __syncthreads();
    if (mine) {
      const double f = !staged ? prod[threadIdx.x] : (myLen > 0 ? prod[sStart[threadIdx.x] - base] : 0.0);
      fl.F(comp)[off] = f;
      if (MODE == 0) {
        put_mirrored<WALLS>(fl.U(comp), g, comp, i, j, k, uOld + g.dt * (f - fo));
        fCur[myR] = f;
      } else {
        fPrev[myR] = fo;
        fCur[myR] = f;
      }
    }
    __syncthreads();
  }
}

template <int MODE, bool WALLS, int FIRST = 0>
__global__ void __launch_bounds__(kSpreadBlock, 2048 / kSpreadBlock) k_spread(Geom g, const Counters* cnt, const int* __restrict__ runStart,
                                                   const int* __restrict__ runCnt,
                                                   const uint32_t* __restrict__ runKey,
                                                   const uint32_t* __restrict__ planRoot,
                                                   const double* __restrict__ planW, const double* __restrict__ fv,
                                                   int cap, Fields fl, double* fCur, double* fPrev, int onlyComp) {
  // prod: the staged products; a node's sum replaces its first product (a node
  // without products keeps 0), and without staging prod[t] holds node t's sum
  extern __shared__ double prod[];
  __shared__ int bins[kLenBins];
  __shared__ int order[kSpreadBlock];
  __shared__ int sStart[kSpreadBlock + 1];  // the block's runs are contiguous: run t spans sStart[t]..sStart[t+1]
  spread_chunks<MODE, WALLS, FIRST>(g, cnt, runStart, runCnt, runKey, planRoot, planW, fv, cap, fl, fCur, fPrev,
                                    onlyComp, blockIdx.x, gridDim.x, prod, bins, order, sStart);
}
constexpr size_t kSpreadSmem = sizeof(double) * kSpreadBuf;


// ---- the forcing loop of many cases in shared launches ----------------------
// A batch of independent cases runs each forcing iteration as two launches for
// all of its members (interpolation, then spreading with the post-guess)
// instead of two per member.  Every block finds its member in a table of block
// owners that follows the members' descriptors, copies the member's
// descriptor into shared memory, and runs the same per-block code as the
// per-case kernels on that member's state, so each member's results are the
// ones it gets alone.
struct MemberDesc {
  Geom g;
  Recs R;
  Fields fl;
  const Counters* cnt;
  const double* W;
  const int4* win;
  double* fv;
  const int* runStart;
  const int* runCnt;
  const uint32_t* runKey;
  const uint32_t* planRoot;
  const double* planW;
  double* fCur;
  double* fPrev;
  int interpBlocks, interpStart;  // blocks per velocity component; first block (3 * interpBlocks per member)
  int spreadBlocks, spreadStart;
};

// The table after the descriptors: the member of every interpolation block,
// then of every spread block (one load instead of a search per block).
__device__ inline int member_of(const MemberDesc* __restrict__ D, int n, int b, bool spread, int interpTotal) {
  const int* __restrict__ owner = reinterpret_cast<const int*>(D + n);
  return owner[spread ? interpTotal + b : b];
}

// copy member `mi`'s descriptor into shared memory (the whole block takes part)
__device__ inline void load_member(const MemberDesc* __restrict__ D, int mi, unsigned char* raw) {
  const int* src = reinterpret_cast<const int*>(D + mi);
  int* dst = reinterpret_cast<int*>(raw);
  for (int i = threadIdx.x; i < (int)(sizeof(MemberDesc) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
}

template <int BS>
__global__ void __launch_bounds__(BS) k_interp_batch(const MemberDesc* __restrict__ D, int n, int first) {
  __shared__ __align__(16) unsigned char raw[sizeof(MemberDesc)];
  __shared__ int sMember;
  if (threadIdx.x == 0) sMember = member_of(D, n, blockIdx.x, false, 0);
  __syncthreads();
  load_member(D, sMember, raw);
  __syncthreads();
  const MemberDesc& d = *reinterpret_cast<const MemberDesc*>(raw);
  const int local = blockIdx.x - d.interpStart;
  const int comp = local / d.interpBlocks;
  const int m = (local - comp * d.interpBlocks) * BS + threadIdx.x;
  if (comp > 2 || m >= d.cnt->npLocal) return;
  if (d.g.unit_h)
    interp_one<1>(d.R, d.g, d.W, d.win, d.fl, d.fv, comp, first, m);
  else
    interp_one<0>(d.R, d.g, d.W, d.win, d.fl, d.fv, comp, first, m);
}

// ANYWALL: some member has solid walls (their halo writes take the general
// path); a batch of periodic cases gets the periodic path only
template <int FIRST, bool ANYWALL>
__global__ void __launch_bounds__(kSpreadBlock, 2048 / kSpreadBlock) k_spread_batch(const MemberDesc* __restrict__ D,
                                                                                   int n, int interpTotal) {
  extern __shared__ double prod[];
  __shared__ int bins[kLenBins];
  __shared__ int order[kSpreadBlock];
  __shared__ int sStart[kSpreadBlock + 1];
  __shared__ __align__(16) unsigned char raw[sizeof(MemberDesc)];
  __shared__ int sMember;
  if (threadIdx.x == 0) sMember = member_of(D, n, blockIdx.x, true, interpTotal);
  __syncthreads();
  load_member(D, sMember, raw);
  __syncthreads();
  const MemberDesc& d = *reinterpret_cast<const MemberDesc*>(raw);
  const int lb = blockIdx.x - d.spreadStart;
  if (ANYWALL && d.g.anyWall)
    spread_chunks<0, true, FIRST>(d.g, d.cnt, d.runStart, d.runCnt, d.runKey, d.planRoot, d.planW, d.fv, d.R.cap,
                                  d.fl, d.fCur, d.fPrev, -1, lb, d.spreadBlocks, prod, bins, order, sStart);
  else
    spread_chunks<0, false, FIRST>(d.g, d.cnt, d.runStart, d.runCnt, d.runKey, d.planRoot, d.planW, d.fv, d.R.cap,
                                   d.fl, d.fCur, d.fPrev, -1, lb, d.spreadBlocks, prod, bins, order, sStart);
}

// VelocityPostGuess (fluid.F90:135-153) + halo refill, per touched node
template <bool WALLS>
__global__ void k_post_guess(Geom g, const Counters* cnt, const uint32_t* runKey, Fields fl, const double* fCur,
                             const double* fPrev) {
  const long long nRuns = cnt->nRuns;
  GRID_STRIDE(r, nRuns) {
    int comp, i, j, k;
    node_coords(g, runKey[r], comp, i, j, k);
    double* U = fl.U(comp);
    long long off = field_off(g, i, j, k);
    put_mirrored<WALLS>(U, g, comp, i, j, k, U[off] + g.dt * (fCur[r] - fPrev[r]));
  }
}

__global__ void k_record_written(Counters* cnt, const uint32_t* runKey, uint32_t* lastNodes) {
  const long long n = cnt->nRuns;
  GRID_STRIDE(t, n) lastNodes[t] = runKey[t];
  if (blockIdx.x == 0 && threadIdx.x == 0) cnt->nLast = (int)n;
}

Fields fields_of(Ctx& c) { return Fields{c.u, c.v, c.w, c.u0, c.v0, c.w0, c.fx, c.fy, c.fz}; }

}  // namespace

static size_t touch_bytes(const Ctx& c) { return (size_t)((3 * c.g.nint + 127) / 128) * 16; }

void launch_weights(Ctx& c, bool locals) {
  int n = locals ? c.capLocal : c.capImg;
  if (n <= 0) return;
  // the locals' launch starts the touched-node bits afresh, the images' adds
  // to them; a plan built after exactly that pair uses them as they are
  unsigned* touch = reinterpret_cast<unsigned*>(c.touch);
  if (locals) cudaMemsetAsync(c.touch, 0, touch_bytes(c), c.stream);
  if (c.g.unit_h)
    k_weights<1><<<nblocks(n), kBlock, 0, c.stream>>>(c.rec(), c.g, c.dCnt, locals, c.W, c.win, c.cntInt, touch);
  else
    k_weights<0><<<nblocks(n), kBlock, 0, c.stream>>>(c.rec(), c.g, c.dCnt, locals, c.W, c.win, c.cntInt, touch);
  c.launches++;
  c.touchState = locals ? 1 : (c.touchState == 1 ? 2 : 0);
}

// touched-node flags, their per-block counts (iTmpA, scanned) and the total (dTotal)
static void flag_touched_nodes(Ctx& c, cudaStream_t s) {
  const long long nvec = (3 * c.g.nint + 127) / 128;
  k_win_by_cell<<<nblocks(c.cap), kBlock, 0, s>>>(c.dCnt, c.cellItems, c.win, c.winC);
  c.launches++;
  if (c.touchState != 2) {
    // the weights were not made as a locals-then-images pair since the bits
    // were last cleared: mark every window again
    cudaMemsetAsync(c.touch, 0, touch_bytes(c), s);
    k_touch<<<nblocks(c.cap), kBlock, 0, s>>>(c.g, c.dCnt, c.winC, reinterpret_cast<unsigned*>(c.touch));
    c.launches++;
  }
  const long long nb = nblocks(nvec);
  k_flag_count<<<(unsigned)nb, kBlock, 0, s>>>(reinterpret_cast<const uint4*>(c.touch), nvec, c.iTmpA);
  scan_exclusive(c.iTmpA, c.iTmpA, nb, nullptr, c.dTotal, c.scanScratch, s, &c.launches);
  c.launches++;
}

long long count_touched_nodes(Ctx& c) {
  flag_touched_nodes(c, c.stream);
  int total = 0;
  if (cudaMemcpyAsync(&total, c.dTotal, sizeof total, cudaMemcpyDeviceToHost, c.stream) != cudaSuccess ||
      cudaStreamSynchronize(c.stream) != cudaSuccess)
    return -1;
  return total;
}

// Grid of the plan fill and the spread: one block per kBlock touched nodes of
// the count the host last read back, plus an eighth (blocks past the device's
// count return at once; the kernels' grid-stride loops cover growth beyond it).
// One batch per block, rather than a resident grid looping over batches, lets
// blocks start as others finish: their load and FP64 phases interleave and no
// block's run of heavy batches holds up the end of the launch.
static int run_blocks(const Ctx& c, int per = kBlock) {
  const long long n = c.runsSeen > 0 ? std::min(c.capRuns, c.runsSeen + c.runsSeen / 8 + kBlock) : c.capRuns;
  return std::max(nblocks(n, per), 1);
}

void build_spread_plan(Ctx& c) {
  cudaStream_t s = c.stream;
  const long long nflags = 3 * c.g.nint;
  const long long nvec = (nflags + 127) / 128;
  flag_touched_nodes(c, s);
  const uint4* fv4 = reinterpret_cast<const uint4*>(c.touch);
  const long long nb = nblocks(nvec);
  k_set_runs<<<1, 1, 0, s>>>(c.dCnt, c.dTotal, c.capRuns);
  k_flag_emit<<<(unsigned)nb, kBlock, 0, s>>>(fv4, nvec, nflags, c.iTmpA, c.runKey, c.capRuns, c.dCnt, c.g.nint);
  cudaMemsetAsync(c.planAlloc, 0, sizeof(unsigned long long), s);
  c.launches += 2;
  k_plan_fill<<<run_blocks(c), kBlock, 0, s>>>(c.g, c.dCnt, c.runKey, c.cellStart, c.cellItems, c.winC, c.W,
                                                   c.imgSrc, c.runStart, c.runCnt, c.planRoot, c.planW, c.planAlloc,
                                                   c.capContrib);
  k_plan_total<<<1, 1, 0, s>>>(c.dCnt, c.planAlloc);
  c.launches += 2;
  c.planReady = true;
  c.spreadValid = false;
}

void launch_mdf_reset(Ctx& c, bool frozen) {
  long long n = std::max<long long>(c.capRuns, c.capLocal);
  auto k = c.g.anyWall ? k_mdf_reset<true> : k_mdf_reset<false>;
  k<<<gs_blocks(n), kBlock, 0, c.stream>>>(c.rec(), c.g, c.dCnt, fields_of(c), c.lastNodes, c.fCur, frozen ? 1 : 0);
  c.launches++;
  c.spreadValid = true;
}

void launch_interp(Ctx& c, int comp, int first) {
  dim3 grid(nblocks(c.capLocal), comp < 0 ? 3 : 1);
  const int comp0 = comp < 0 ? 0 : comp;
  auto k = c.g.unit_h ? k_interp<1> : k_interp<0>;
  k<<<grid, kBlock, 0, c.stream>>>(c.rec(), c.g, c.dCnt, c.W, c.win, fields_of(c), c.fv, comp0, first);
  c.launches++;
}

// the spread with the post-guess fused (MODE 0) or keeping fx and fxOld for a
// separate VelocityPostGuess (MODE 1); the halo writes know about walls only
// when the case has some
void launch_spread(Ctx& c, bool fused_post_guess, int comp, int first) {
  const bool w = c.g.anyWall;
  using K = void (*)(Geom, const Counters*, const int*, const int*, const uint32_t*, const uint32_t*, const double*,
                     const double*, int, Fields, double*, double*, int);
  K k;
  if (!fused_post_guess)
    k = w ? k_spread<1, true> : k_spread<1, false>;
  else if (first == 3)
    k = w ? k_spread<0, true, 3> : k_spread<0, false, 3>;
  else if (first == 1)
    k = w ? k_spread<0, true, 1> : k_spread<0, false, 1>;
  else
    k = w ? k_spread<0, true> : k_spread<0, false>;
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSpreadSmem);
  // one component: about a third of the runs, plus the block across its start
  const int nb = run_blocks(c, kSpreadBlock);
  const int grid = comp < 0 ? nb : std::max(1, (nb + 2) / 3 + 1);
  k<<<grid, kSpreadBlock, kSpreadSmem, c.stream>>>(c.g, c.dCnt, c.runStart, c.runCnt, c.runKey, c.planRoot, c.planW, c.fv,
                                             c.cap, fields_of(c), c.fCur, c.fPrev, comp);
  c.launches++;
}

void launch_mdf_stale(Ctx& c, bool frozen) {
  auto k = c.g.anyWall ? k_mdf_stale<true> : k_mdf_stale<false>;
  k<<<gs_blocks(c.capRuns), kBlock, 0, c.stream>>>(c.g, c.dCnt, fields_of(c), c.lastNodes,
                                                   reinterpret_cast<const unsigned*>(c.touch), frozen ? 1 : 0);
  c.launches++;
  c.spreadValid = true;
}

// blocks of a member: per velocity component for the interpolation, in all
// for the spread (the per-case launches' grids)
static int interp_blocks_of(const Ctx& c, int interpBlock) { return nblocks(std::max(c.capLocal, 1), interpBlock); }

size_t forcing_desc_bytes(const std::vector<Ctx*>& members, int interpBlock) {
  size_t blocks = 0;
  for (const Ctx* c : members) blocks += 3 * (size_t)interp_blocks_of(*c, interpBlock) + run_blocks(*c, kSpreadBlock);
  return sizeof(MemberDesc) * std::max<size_t>(members.size(), 1) + sizeof(int) * blocks;
}

cudaError_t forcing_desc_upload(const std::vector<Ctx*>& members, void* dDesc, int interpBlock, cudaStream_t s,
                                ForcingBatch* fb) {
  const size_t n = members.size();
  std::vector<MemberDesc> h(n);
  int ib = 0, sb = 0;
  for (size_t q = 0; q < n; ++q) {
    Ctx& c = *members[q];
    MemberDesc& d = h[q];
    d.g = c.g;
    d.R = c.rec();
    d.fl = fields_of(c);
    d.cnt = c.dCnt;
    d.W = c.W;
    d.win = c.win;
    d.fv = c.fv;
    d.runStart = c.runStart;
    d.runCnt = c.runCnt;
    d.runKey = c.runKey;
    d.planRoot = c.planRoot;
    d.planW = c.planW;
    d.fCur = c.fCur;
    d.fPrev = c.fPrev;
    d.interpBlocks = interp_blocks_of(c, interpBlock);
    d.interpStart = ib;
    ib += 3 * d.interpBlocks;
    d.spreadBlocks = run_blocks(c, kSpreadBlock);
    d.spreadStart = sb;
    sb += d.spreadBlocks;
  }
  std::vector<int> owner((size_t)ib + sb);
  for (size_t q = 0; q < n; ++q) {
    std::fill(owner.begin() + h[q].interpStart, owner.begin() + h[q].interpStart + 3 * h[q].interpBlocks, (int)q);
    std::fill(owner.begin() + ib + h[q].spreadStart,
              owner.begin() + ib + h[q].spreadStart + h[q].spreadBlocks, (int)q);
  }
  fb->desc = dDesc;
  fb->n = (int)n;
  fb->interpBlocksTotal = ib;
  fb->spreadBlocksTotal = sb;
  fb->interpBlock = interpBlock;
  fb->anyWall = false;
  for (Ctx* c : members) fb->anyWall = fb->anyWall || c->g.anyWall;
  char* base = static_cast<char*>(dDesc);
  cudaError_t e = cudaMemcpyAsync(base, h.data(), sizeof(MemberDesc) * n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && !owner.empty())
    e = cudaMemcpyAsync(base + sizeof(MemberDesc) * n, owner.data(), sizeof(int) * owner.size(),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e;
}

void launch_forcing_batch(const ForcingBatch& fb, int first, cudaStream_t s) {
  const MemberDesc* D = static_cast<const MemberDesc*>(fb.desc);
  if (fb.interpBlock == 128)
    k_interp_batch<128><<<fb.interpBlocksTotal, 128, 0, s>>>(D, fb.n, first);
  else
    k_interp_batch<kBlock><<<fb.interpBlocksTotal, kBlock, 0, s>>>(D, fb.n, first);
  auto k = first == 3 ? (fb.anyWall ? k_spread_batch<3, true> : k_spread_batch<3, false>)
                      : (fb.anyWall ? k_spread_batch<0, true> : k_spread_batch<0, false>);
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSpreadSmem);
  k<<<fb.spreadBlocksTotal, kSpreadBlock, kSpreadSmem, s>>>(D, fb.n, fb.interpBlocksTotal);
}

void launch_post_guess(Ctx& c) {
  auto k = c.g.anyWall ? k_post_guess<true> : k_post_guess<false>;
  k<<<gs_blocks(c.capRuns), kBlock, 0, c.stream>>>(c.g, c.dCnt, c.runKey, fields_of(c), c.fCur, c.fPrev);
  c.launches++;
}

void record_written_nodes(Ctx& c) {
  k_record_written<<<gs_blocks(c.capRuns), kBlock, 0, c.stream>>>(c.dCnt, c.runKey, c.lastNodes);
  c.launches++;
}


// ---- interpolation at caller-given points, without allocation ---------------
// Some callers sample the fluid at probe points from inside their own time
// loop, where they must not allocate device memory: a fluid solver that has
// committed the device memory to its own arrays (an allocation there can fail
// in the middle of a run), or one that keeps other streams busy while the
// particles advance (cudaMalloc and cudaFree synchronise the whole device).
// This variant of the weight and interpolation kernels keeps the per-point
// weights and windows in one fixed static device array instead of context
// buffers, so a call allocates nothing.  The array is shared by every call on
// a device: calls that overlap in time race on it.

constexpr size_t kProbeWBytes = (size_t)IBMDEM_PROBE_MAX_POINTS * kWStride * sizeof(double);
constexpr size_t kProbeWinBytes = (size_t)IBMDEM_PROBE_MAX_POINTS * sizeof(int4);
constexpr size_t kProbeScratchBytes = kProbeWBytes + kProbeWinBytes + 256;
static_assert(kProbeWBytes % 256 == 0 && kProbeWinBytes % 256 == 0, "sections start on 256-byte boundaries");
constexpr int kProbeMaxDevices = 64;

// weights (kWStride doubles per point) | windows (int4 per point) | status
// word; about 11.3 MB for 16384 points.
static __device__ __align__(256) unsigned char g_probeScratch[kProbeScratchBytes];

namespace {

std::mutex g_probeMutex;
void* g_probeBase[kProbeMaxDevices] = {};

// k_weights for n caller-given points.  A point's cell is floor((x-xStart)/dx)+1
// per axis, as the cell lists compute it.  A point outside the box (or NaN)
// gets no window and raises *status to n - index, so that the lowest offending
// index is n - *status (*status stays 0 when every point is inside).
template <int UNIT_H>
__global__ void __launch_bounds__(kBlock) k_probe_weights(Geom g, int n, const double* __restrict__ x, double* W,
                                                          int4* win, int* status) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  double xp[3];
  int a[3];
  bool in = true;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    xp[d] = x[(size_t)3 * e + d];
    const double t = floor((xp[d] - g.start[d]) / g.h[d]);
    in = in && t >= 0.0 && t < (double)g.n[d];
    a[d] = in ? (int)t + 1 : 1;
  }
  if (!in) {
    atomicMax(status, n - e);
    win[e] = make_int4(0, 0, 0, -1);
    return;
  }
  double wu[3][3], ws[3][3];
  int flags = 0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const double h = g.h[d];
    double dl[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      double xc = ((double)(a[d] - 1 + q) - 0.5);
      if (!UNIT_H) xc = xc * h;
      dl[q] = xp[d] - xc;
    }
    delta_triple<UNIT_H>(dl, h, wu[d]);
    const double s0 = dl[0] + g.halfh[d];
    const int st = fabs(UNIT_H ? s0 : s0 / h) < 1.5 ? 0 : 1;
    flags |= st << d;
    double xs[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) xs[q] = (st ? dl[q + 1] : dl[q]) + g.halfh[d];
    delta_triple<UNIT_H>(xs, h, ws[d]);
  }
  double4_32a* out = reinterpret_cast<double4_32a*>(W + (size_t)e * kWStride);
#pragma unroll
  for (int comp = 0; comp < 3; ++comp) {
    double wc[28];
#pragma unroll
    for (int ky = 0; ky < 3; ++ky)
#pragma unroll
      for (int kx = 0; kx < 3; ++kx) {
        const double w12 = (comp == 0 ? ws[0][kx] : wu[0][kx]) * (comp == 1 ? ws[1][ky] : wu[1][ky]);
#pragma unroll
        for (int kz = 0; kz < 3; ++kz) {
          double wt = w12 * (comp == 2 ? ws[2][kz] : wu[2][kz]);
          if (!UNIT_H) wt = wt / g.hprod;
          wc[kz * 9 + ky * 3 + kx] = wt;
        }
      }
    wc[27] = 0.0;
#pragma unroll
    for (int q = 0; q < 7; ++q) out[comp * 7 + q] = make_double4_32a(wc[4 * q], wc[4 * q + 1], wc[4 * q + 2], wc[4 * q + 3]);
  }
  win[e] = make_int4(a[0], a[1], a[2], flags);
}

// k_interp's sum for the points (blockIdx.y = component); ulp is (u,v,w) per
// point, NaN for a point outside the box.
template <int UNIT_H>
__global__ void __launch_bounds__(kBlock) k_probe_interp(Geom g, int n, const double* __restrict__ W,
                                                         const int4* __restrict__ win, Fields fl, double* ulpOut) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  const int comp = blockIdx.y;
  const int4 wn = win[m];
  if (wn.w < 0) {
    ulpOut[(size_t)3 * m + comp] = __longlong_as_double(0x7ff8000000000000ll);
    return;
  }
  const double* __restrict__ F = fl.U(comp);
  int sx, sy, sz;
  window_start(wn, comp, sx, sy, sz);
  const double* Wc = W + (size_t)m * kWStride + comp * 28;
  double ulp = 0.0;
#pragma unroll
  for (int kz = 0; kz < 3; ++kz)
#pragma unroll
    for (int ky = 0; ky < 3; ++ky) {
      const double* row = F + field_off(g, sx, sy + ky, sz + kz);
#pragma unroll
      for (int kx = 0; kx < 3; ++kx) {
        double t = Wc[kz * 9 + ky * 3 + kx] * row[kx];
        if (!UNIT_H) {
          t = t * g.h[0];
          t = t * g.h[1];
          t = t * g.h[2];
        }
        ulp = ulp + t;
      }
    }
  ulpOut[(size_t)3 * m + comp] = ulp;
}

}  // namespace

cudaError_t interpolate_points_noalloc(Ctx& c, int n, const double* x, double* ulp, int* bad) {
  *bad = -1;
  if (n < 0 || n > IBMDEM_PROBE_MAX_POINTS) return cudaErrorInvalidValue;
  if (c.device < 0 || c.device >= kProbeMaxDevices) return cudaErrorInvalidDevice;
  void* base = nullptr;
  {
    // Setup, once per device, with that device current (the caller set it):
    // the address of the static array on this device.  The first call may load
    // the module, so it belongs before any stream capture.
    std::lock_guard<std::mutex> lock(g_probeMutex);
    base = g_probeBase[c.device];
    if (!base) {
      const cudaError_t e = cudaGetSymbolAddress(&base, g_probeScratch);
      if (e != cudaSuccess) return e;
      g_probeBase[c.device] = base;
    }
  }
  unsigned char* s = static_cast<unsigned char*>(base);
  double* W = reinterpret_cast<double*>(s);
  int4* win = reinterpret_cast<int4*>(s + kProbeWBytes);
  int* status = reinterpret_cast<int*>(s + kProbeWBytes + kProbeWinBytes);
  // The status word is the one part of the array that must start at zero;
  // every weight and window a call reads is written by that call first.
  cudaError_t e = cudaMemsetAsync(status, 0, sizeof(int), c.stream);
  if (e != cudaSuccess) return e;
  if (n > 0) {
    const dim3 grid(nblocks(n), 3);
    if (c.g.unit_h) {
      k_probe_weights<1><<<nblocks(n), kBlock, 0, c.stream>>>(c.g, n, x, W, win, status);
      k_probe_interp<1><<<grid, kBlock, 0, c.stream>>>(c.g, n, W, win, fields_of(c), ulp);
    } else {
      k_probe_weights<0><<<nblocks(n), kBlock, 0, c.stream>>>(c.g, n, x, W, win, status);
      k_probe_interp<0><<<grid, kBlock, 0, c.stream>>>(c.g, n, W, win, fields_of(c), ulp);
    }
    c.launches += 2;
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  int h = 0;
  e = cudaMemcpyAsync(&h, status, sizeof h, cudaMemcpyDeviceToHost, c.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
  if (e != cudaSuccess) return e;
  if (h > 0) *bad = n - h;
  return cudaSuccess;
}

}  // namespace ibmdem
