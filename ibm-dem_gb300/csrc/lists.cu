// lists.cu — RebuildParcelInCellListDEM on the GPU (ZJS_UPDATE_LIST_DEM.F90:2-177).
//
// The reference drops parcels that left the domain (CompressDEM), bins the
// rest into cells in part order, and exchanges 2-cell halo layers face by face
// (x, then y, then z) so that periodic images of parcels, edges and corners
// included, are appended behind the locals.  The order of those images is
// fixed by the face loop: all images of one (x,y,z) shift class are contiguous,
// classes come in the order the face loop creates them, and inside a class the
// sources keep their part order.  Here every local parcel derives its image
// classes from its cell and one class-major scan places all images at once.
#include "common.cuh"
#include "kernels.cuh"
#include "prims.cuh"

namespace ibmdem {

namespace {

// ---- CompressDEM (ZJS_UPDATE_LIST_DEM.F90:2-27) ------------------------------
__global__ void k_compress_flags(Recs R, Geom g, const Counters* cnt, int* flag) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= cnt->np) return;
  int a = cell_of(g, 0, R.D(D_X, e));
  int b = cell_of(g, 1, R.D(D_X + 1, e));
  int c = cell_of(g, 2, R.D(D_X + 2, e));
  flag[e] = interior(g, a, b, c) ? 1 : 0;
}

// The compaction runs in place.  A kept parcel whose slot does not change (all
// the locals, unless one left the interior) only gets its cell index; the
// others -- kept parcels behind a dropped one -- go to their new slot through
// the spare record set in two passes (a new slot can hold a parcel that moves
// too).  No kept parcel that stays is a destination: a parcel stays only when
// every parcel before it is kept, and then every later kept parcel lands after it.
__device__ inline void set_cell(Recs R, const Geom& g, int n) {
  int a = cell_of(g, 0, R.D(D_X, n));
  int b = cell_of(g, 1, R.D(D_X + 1, n));
  int c = cell_of(g, 2, R.D(D_X + 2, n));
  R.I(I_CELL, n) = cell_id(g, a, b, c);
}

__device__ inline void copy_record(Recs A, int e, Recs B, int n) {
#pragma unroll
  for (int f = 0; f < ND; ++f) B.D(f, n) = A.D(f, e);
  B.I(I_GIDX, n) = A.I(I_GIDX, e);
  B.I(I_MSIDX, n) = A.I(I_MSIDX, e);
  B.I(I_PID, n) = A.I(I_PID, e);
}

__global__ void k_compress_move(Recs A, Recs B, Geom g, const Counters* cnt, const int* flag, const int* pos) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= cnt->np || !flag[e]) return;
  const int n = pos[e];
  if (n == e)
    set_cell(A, g, e);
  else
    copy_record(A, e, B, n);
}

__global__ void k_compress_back(Recs A, Recs B, Geom g, const Counters* cnt, const int* flag, const int* pos) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= cnt->np || !flag[e]) return;
  const int n = pos[e];
  if (n == e) return;
  copy_record(B, n, A, n);
  set_cell(A, g, n);
}

__global__ void k_set_local_counts(Counters* cnt, const int* total) {
  int n = *total;
  cnt->npLocal = n;
  cnt->np = n;
  cnt->nImg = 0;
}

// ---- periodic and wall images -------------------------------------------------
// Variant code per axis: 0 none; 1 = the image the face loop makes beyond the
// high face, 2 = beyond the low face.  On a periodic axis those are the parcels
// near the low face shifted by +L (1) and near the high face shifted by -L (2)
// (ZJS_UPDATE_LIST_DEM.F90:147-151).  Across solid walls there is no rank to
// send to, and UpdateFullInfoForSolidOutletBoundary (ZJS_MPI_DEM.F90:173-210)
// mirrors the parcels near the receiving face about it instead: near the high
// face about the high wall (1), near the low face about the low wall (2), the
// normal velocity negated, pType 1.  Class order of the face loop:
//   0: (+,0,0)  1: (-,0,0)
//   2..4:  sy=+ with sx = 0,+,-     5..7:  sy=- with sx = 0,+,-
//   8..16: sz=+ with (sy,sx) in {0,+,-}^2 (sy major)   17..25: sz=-
constexpr int kClasses = 26;

__device__ inline int class_of(int fx, int fy, int fz) {
  if (fz) return 8 + (fz == 2 ? 9 : 0) + 3 * fy + fx;
  if (fy) return 2 + (fy == 2 ? 3 : 0) + fx;
  return fx == 1 ? 0 : 1;
}

__device__ inline unsigned image_mask(const Geom& g, int a, int b, int c) {
  int opt[3][2];
  int cnt[3];
  int id[3] = {a, b, c};
  for (int d = 0; d < 3; ++d) {
    cnt[d] = 0;
    const bool lo = id[d] >= 1 && id[d] <= kHalo, hi = id[d] >= g.n[d] - kHalo + 1 && id[d] <= g.n[d];
    if (g.wall[d] ? hi : lo) opt[d][cnt[d]++] = 1;
    if (g.wall[d] ? lo : hi) opt[d][cnt[d]++] = 2;
  }
  unsigned m = 0;
  for (int iz = -1; iz < cnt[2]; ++iz)
    for (int iy = -1; iy < cnt[1]; ++iy)
      for (int ix = -1; ix < cnt[0]; ++ix) {
        int fx = ix < 0 ? 0 : opt[0][ix], fy = iy < 0 ? 0 : opt[1][iy], fz = iz < 0 ? 0 : opt[2][iz];
        if (fx | fy | fz) m |= 1u << class_of(fx, fy, fz);
      }
  return m;
}

__device__ inline void class_shift(int cls, int& fx, int& fy, int& fz) {
  if (cls >= 8) {
    int q = cls - 8;
    fz = q >= 9 ? 2 : 1;
    q %= 9;
    fy = q / 3;
    fx = q % 3;
  } else if (cls >= 2) {
    int q = cls - 2;
    fz = 0;
    fy = q >= 3 ? 2 : 1;
    fx = q % 3;
  } else {
    fz = fy = 0;
    fx = cls == 0 ? 1 : 2;
  }
}

// coordinate d of the image of class code s (1, 2) of x: a periodic shift, or
// x(dim) = 2*coordMirror - x(dim) across a wall (ZJS_MPI_DEM.F90:198)
__device__ inline double image_coord(const Geom& g, int d, int s, double x) {
  if (g.wall[d]) return 2.0 * (s == 1 ? g.end[d] : g.start[d]) - x;
  return s == 1 ? x + g.len[d] : x + (-g.len[d]);
}

__device__ inline unsigned local_mask(const Recs& R, const Geom& g, int m) {
  int a, b, c;
  cell_coords(g, R.I(I_CELL, m), a, b, c);
  return image_mask(g, a, b, c);
}

// a warp's image count per class into wc[0..kClasses) (lane 0 writes); only the
// classes some lane of the warp has are balloted (most warps have none).
// Returns the union of the lanes' class masks.
__device__ inline unsigned warp_class_counts(unsigned mask, int lane, int* wc) {
  const unsigned wmask = __reduce_or_sync(0xffffffffu, mask);
  if (lane < kClasses) wc[lane] = 0;
  __syncwarp();
  for (unsigned rest = wmask; rest; rest &= rest - 1u) {
    const int c = __ffs(rest) - 1;
    const unsigned bal = __ballot_sync(0xffffffffu, (mask >> c) & 1u);
    if (lane == 0) wc[c] = __popc(bal);
  }
  return wmask;
}

__global__ void k_img_count(Recs R, Geom g, const Counters* cnt, int* blockCls, long long nb) {
  __shared__ int wc[kBlock / 32][kClasses];
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned mask = m < cnt->npLocal ? local_mask(R, g, m) : 0u;
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  warp_class_counts(mask, lane, wc[warp]);
  __syncthreads();
  if (threadIdx.x < kClasses) {
    int s = 0;
    for (int w = 0; w < kBlock / 32; ++w) s += wc[w][threadIdx.x];
    blockCls[(long long)threadIdx.x * nb + blockIdx.x] = s;
  }
}

__global__ void __launch_bounds__(kBlock, 4) k_img_emit(Recs R, Geom g, Counters* cnt, const int* offs, long long nb, int* imgSrc,
                           int* imgShift, int capImg) {
  __shared__ int wc[kBlock / 32][kClasses];
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  int npLocal = cnt->npLocal;
  unsigned mask = m < npLocal ? local_mask(R, g, m) : 0u;
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned lt = (1u << lane) - 1u;
  const unsigned wmask = warp_class_counts(mask, lane, wc[warp]);
  __syncthreads();
  if (threadIdx.x < kClasses) {
    int run = 0;
    for (int w = 0; w < kBlock / 32; ++w) {
      int t = wc[w][threadIdx.x];
      wc[w][threadIdx.x] = run;
      run += t;
    }
  }
  __syncthreads();
  if (!wmask) return;  // the whole warp: no images
  const int cap = R.cap;
  for (unsigned rest = wmask; rest; rest &= rest - 1u) {
    const int c = __ffs(rest) - 1;
    const unsigned bal = __ballot_sync(0xffffffffu, (mask >> c) & 1u);
    if (!((mask >> c) & 1u)) continue;
    int pos = offs[(long long)c * nb + blockIdx.x] + wc[warp][c] + __popc(bal & lt);
    int e = npLocal + pos;
    if (pos >= capImg || e >= cap) {
      set_err(cnt, E_IMGCAP, e);
      continue;
    }
    int fx, fy, fz;
    class_shift(c, fx, fy, fz);
    int sh[3] = {fx, fy, fz};
#pragma unroll 2
    for (int f = 0; f < ND; ++f) R.D(f, e) = R.D(f, m);
    R.I(I_GIDX, e) = R.I(I_GIDX, m);
    R.I(I_MSIDX, e) = R.I(I_MSIDX, m);
    R.I(I_PID, e) = R.I(I_PID, m);
    int id[3];
    int wallImg = 0;
    // MyMPISendAndRecv does not send vgap and wdrag (ZJS_MPI_DEM.F90:17-32); the
    // slot's leftovers in the reference, zero here (a mirror across a wall copies
    // the whole record, ZJS_MPI_DEM.F90:194, and takes them back below)
#pragma unroll
    for (int d = 0; d < 3; ++d) R.D(D_VGAP + d, e) = 0.0;
    R.D(D_WDRAG, e) = 0.0;
    for (int d = 0; d < 3; ++d) {
      double x = R.D(D_X + d, m);
      if (sh[d]) {
        x = image_coord(g, d, sh[d], x);
        if (g.wall[d]) {
          R.D(D_V + d, e) = -R.D(D_V + d, m);
          wallImg = 1;
        }
      }
      R.D(D_X + d, e) = x;
      id[d] = cell_of(g, d, x);
    }
    R.I(I_CELL, e) = cell_id(g, id[0], id[1], id[2]);
    // a chain of mirrors keeps the source's values; a periodic step in it zeroes them
    bool allWall = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) allWall = allWall && (!sh[d] || g.wall[d]);
    if (allWall) {
#pragma unroll
      for (int d = 0; d < 3; ++d) R.D(D_VGAP + d, e) = R.D(D_VGAP + d, m);
      R.D(D_WDRAG, e) = R.D(D_WDRAG, m);
    }
    imgSrc[pos] = m;
    imgShift[pos] = fx | (fy << 2) | (fz << 4) | (wallImg << kWallImgBit);
  }
}

__global__ void k_set_image_counts(Counters* cnt, const int* total, int capImg) {
  int n = *total;
  if (n > capImg) {
    atomicOr(&cnt->err, E_IMGCAP);
    cnt->errInfo = n;
    n = capImg;
  }
  cnt->nImg = n;
  cnt->np = cnt->npLocal + n;
}

// ---- UpdateParcelInfoInGhostRegion (ZJS_UPDATE_LIST_DEM.F90:179-246; across
// walls UpdatePartInfoForSolidOutletBoundary, ZJS_MPI_DEM.F90:222-269) -------
__global__ void k_img_update(Recs R, Geom g, const Counters* cnt, const int* imgSrc, const int* imgShift) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= cnt->nImg) return;
  int e = cnt->npLocal + q;
  int m = imgSrc[q];
  int code = imgShift[q];
  R.I(I_MSIDX, e) = R.I(I_MSIDX, m);
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    int s = (code >> (2 * d)) & 3;
    double x = R.D(D_X + d, m);
    const double v = R.D(D_V + d, m);
    if (s) x = image_coord(g, d, s, x);
    R.D(D_X + d, e) = x;
    // across a wall the normal velocity is negated (ZJS_MPI_DEM.F90:256); fdrag is copied as is
    R.D(D_V + d, e) = (s && g.wall[d]) ? -v : v;
    R.D(D_FDRAG + d, e) = R.D(D_FDRAG + d, m);
  }
  R.D(D_WSUM, e) = R.D(D_WSUM, m);
}

// ---- cell and body lists -----------------------------------------------------
// The cell lists (npPartInCell / partIdxInCell) without a sort: a parcel takes
// a slot in its cell from the count's atomic, the exclusive scan of the counts
// gives the cells' starts, the parcels scatter to start + slot, and the parcel
// that took slot 0 puts its cell's few items back in part order -- the order a
// stable sort by cell gives.
__global__ void k_cell_keys(Recs R, Geom g, Counters* cnt, uint32_t* cellOf, int* slot, int* cellCount) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= cnt->np) return;
  int id = R.I(I_CELL, e);
  if (id < 1 || id > g.ncell) {
    set_err(cnt, E_RANGE, e);
    id = 1;
  }
  cellOf[e] = (uint32_t)(id - 1);
  slot[e] = atomicAdd(&cellCount[id - 1], 1);
}

// parcel e to its cell's start + slot; the cell's count goes back to zero
// for the next rebuild
__global__ void k_cell_scatter(const Counters* cnt, const uint32_t* __restrict__ cellOf, const int* __restrict__ slot,
                               const int* __restrict__ cellStart, int* cellItems, int* cellCount) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= cnt->np) return;
  const uint32_t c = cellOf[e];
  cellItems[cellStart[c] + slot[e]] = e;
  if (slot[e] == 0) cellCount[c] = 0;
}

// Shell sort (Ciura's gaps) of a cell's items: an insertion sort for the usual
// handful, and no quadratic cost for a cell that holds very many parcels
__global__ void k_cell_order(const Counters* cnt, const uint32_t* __restrict__ cellOf, const int* __restrict__ slot,
                             const int* __restrict__ cellStart, int* cellItems) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= cnt->np || slot[e] != 0) return;
  const uint32_t c = cellOf[e];
  const int s = cellStart[c], n = cellStart[c + 1] - s;
  if (n < 2) return;
  int* a = cellItems + s;
  constexpr int kGaps[8] = {701, 301, 132, 57, 23, 10, 4, 1};
  for (int gi = 0; gi < 8; ++gi) {
    const int gap = kGaps[gi];
    for (int i = gap; i < n; ++i) {
      const int v = a[i];
      int j = i;
      while (j >= gap && a[j - gap] > v) {
        a[j] = a[j - gap];
        j -= gap;
      }
      a[j] = v;
    }
  }
}

__global__ void k_body_keys(Recs R, Counters* cnt, int nMS, uint32_t* keys, uint32_t* vals, int* bodyCount) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= cnt->npLocal) return;
  int b = R.I(I_MSIDX, m);
  if (b < 1 || b > nMS) {
    set_err(cnt, E_MSIDX, m);
    b = 1;
  }
  keys[m] = (uint32_t)(b - 1);
  vals[m] = (uint32_t)m;
  // a body's markers are mostly neighbours in part order: one atomic per body
  // and warp instead of one per marker on the same counter
  const unsigned peers = __match_any_sync(__activemask(), b);
  if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&bodyCount[b - 1], __popc(peers));
}

int bits_for(long long n) {
  int b = 1;
  while ((1ll << b) < n) ++b;
  return b;
}

}  // namespace

void launch_img_update(Ctx& c) {
  k_img_update<<<nblocks(c.capImg), kBlock, 0, c.stream>>>(c.rec(), c.g, c.dCnt, c.imgSrc, c.imgShift);
  c.launches++;
}

void rebuild_cell_lists(Ctx& c) {
  cudaStream_t s = c.stream;
  // CompressDEM: keep parcels (locals and images) whose cell is interior
  k_compress_flags<<<nblocks(c.cap), kBlock, 0, s>>>(c.rec(), c.g, c.dCnt, c.iTmpA);
  scan_exclusive(c.iTmpA, c.iTmpB, c.cap, &c.dCnt->np, c.dTotal, c.scanScratch, s, &c.launches);
  k_compress_move<<<nblocks(c.cap), kBlock, 0, s>>>(c.rec(), c.recAlt(), c.g, c.dCnt, c.iTmpA, c.iTmpB);
  k_compress_back<<<nblocks(c.cap), kBlock, 0, s>>>(c.rec(), c.recAlt(), c.g, c.dCnt, c.iTmpA, c.iTmpB);
  k_set_local_counts<<<1, 1, 0, s>>>(c.dCnt, c.dTotal);
  c.launches += 4;
  // periodic images, class-major in the face-loop order
  long long nbl = nblocks(c.capLocal);
  k_img_count<<<(unsigned)nbl, kBlock, 0, s>>>(c.rec(), c.g, c.dCnt, c.iTmpA, nbl);
  scan_exclusive(c.iTmpA, c.iTmpA, kClasses * nbl, nullptr, c.dTotal, c.scanScratch, s, &c.launches);
  k_img_emit<<<(unsigned)nbl, kBlock, 0, s>>>(c.rec(), c.g, c.dCnt, c.iTmpA, nbl, c.imgSrc, c.imgShift,
                                                 c.capImg);
  k_set_image_counts<<<1, 1, 0, s>>>(c.dCnt, c.dTotal, c.capImg);
  c.launches += 3;
  // cell lists: stable sort of part indices by cell (npPartInCell/partIdxInCell)
  k_cell_keys<<<nblocks(c.cap), kBlock, 0, s>>>(c.rec(), c.g, c.dCnt, c.kA, c.iTmpA, c.cellCount);
  c.launches++;
  c.planReady = false;  // the plan is rebuilt after new weights
  scan_exclusive(c.cellCount, c.cellStart, c.g.ncell, nullptr, c.cellStart + c.g.ncell, c.scanScratch, s,
                 &c.launches);
  k_cell_scatter<<<nblocks(c.cap), kBlock, 0, s>>>(c.dCnt, c.kA, c.iTmpA, c.cellStart, c.cellItems, c.cellCount);
  k_cell_order<<<nblocks(c.cap), kBlock, 0, s>>>(c.dCnt, c.kA, c.iTmpA, c.cellStart, c.cellItems);
  c.launches += 2;
  uint32_t *k0, *v0, *k1, *v1;
  // body lists for AssembleLocalForceMS: locals grouped by body in part order
  if (c.nMS > 0) {
    cudaMemsetAsync(c.bodyStart, 0, sizeof(int) * (c.nMS + 1), s);
    k_body_keys<<<nblocks(c.capLocal), kBlock, 0, s>>>(c.rec(), c.dCnt, c.nMS, c.kA, c.vA, c.bodyStart);
    c.launches++;
    k0 = c.kA, v0 = c.vA, k1 = c.kB, v1 = c.vB;
    radix_sort_pairs(k0, v0, k1, v1, c.capLocal, &c.dCnt->npLocal, bits_for(c.nMS), c.sortHist, c.scanScratch, s,
                     &c.launches);
    cudaMemcpyAsync(c.bodyItems, v0, sizeof(int) * c.capLocal, cudaMemcpyDeviceToDevice, s);
    scan_exclusive(c.bodyStart, c.bodyStart, c.nMS, nullptr, c.bodyStart + c.nMS, c.scanScratch, s, &c.launches);
  }
}

}  // namespace ibmdem
