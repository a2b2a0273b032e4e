// api.cu — the C ABI of include/ibmdem.h: context lifetime, device allocation,
// record conversion, and the reference-named entry points and drivers.
//
// Work is stream-ordered and issued without host round trips; errors raised
// on the device (capacity, range) are latched in a device word and reported by
// the next call that synchronises (getters, ibmdem_synchronize).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "common.cuh"
#include "kernels.cuh"
#include "prims.cuh"

using namespace ibmdem;

namespace {

int set_error(ibmdem_ctx* h, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (h) h->c.err = buf;
  return code;
}

#define CU(call)                                                                                \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      return set_error(h, IBMDEM_ECUDA, "%s failed: %s", #call, cudaGetErrorString(e_));       \
  } while (0)

// Device memory is stream-ordered (the device's default pool, on the context's
// stream): unlike cudaMalloc/cudaFree, setting up or tearing down one case
// does not serialise the work other cases have in flight on other streams.
template <typename T>
cudaError_t dalloc(Ctx& c, T*& p, size_t n) {
  p = nullptr;
  const size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
  const cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&p), bytes, c.stream);
  if (e == cudaSuccess) c.bytes += bytes;
  return e;
}

void dfree(Ctx& c, void* p) {
  if (p) cudaFreeAsync(p, c.stream);
}

// Keep freed blocks in the device's default pool (a process-local attribute) so
// that cases created after others finished reuse them without new mappings.
void retain_pool_memory(int device) {
  static std::mutex mu;
  static bool done[64] = {};
  std::lock_guard<std::mutex> lock(mu);
  if (device < 0 || device >= 64 || done[device]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  done[device] = true;
}

// Pinned mirrors of the device counters come from shared slabs: a pinned host
// allocation per case would serialise the device like cudaMalloc does.
std::mutex g_pinMutex;
std::vector<Counters*> g_pinFree;

Counters* pinned_counters() {
  std::lock_guard<std::mutex> lock(g_pinMutex);
  if (g_pinFree.empty()) {
    constexpr int kSlab = 256;
    Counters* slab = nullptr;
    if (cudaMallocHost(reinterpret_cast<void**>(&slab), sizeof(Counters) * kSlab) != cudaSuccess) return nullptr;
    for (int i = kSlab - 1; i >= 0; --i) g_pinFree.push_back(slab + i);
  }
  Counters* q = g_pinFree.back();
  g_pinFree.pop_back();
  return q;
}

void release_counters(Counters* q) {
  if (!q) return;
  std::lock_guard<std::mutex> lock(g_pinMutex);
  g_pinFree.push_back(q);
}

double eta_of(double e) {
  // ZJS_COLLISION_DEM.F90:30: 3.1415926536 is a single-precision literal
  float pi32 = 3.1415926536f;
  float pi2 = pi32 * pi32;
  return -2 * std::log(e) / std::sqrt((double)pi2 + std::log(e));
}

void free_history(Ctx& c) {
  void* ps[] = {c.histRange[0], c.histRange[1], c.histGid[0], c.histGid[1], c.histXi[0], c.histXi[1], c.pidMap};
  for (void* p : ps) dfree(c, p);
  c.histRange[0] = c.histRange[1] = nullptr;
  c.histGid[0] = c.histGid[1] = nullptr;
  c.histXi[0] = c.histXi[1] = nullptr;
  c.pidMap = nullptr;
  c.bytes -= c.bytesHist;
  c.bytesHist = 0;
}

void free_parcel_buffers(Ctx& c) {
  free_history(c);
  void* ps[] = {c.recD[0], c.recD[1], c.recI[0], c.recI[1], c.imgSrc, c.imgShift, c.cellItems, c.bodyItems,
                c.iTmpA, c.iTmpB, c.scanScratch, c.sortHist, c.kA, c.vA, c.kB, c.vB, c.activeList, c.pairCnt,
                c.pairStart, c.pairIdx, c.W, c.win, c.cntInt, c.fv, c.runStart, c.runKey, c.fCur, c.fPrev,
                c.lastNodes, c.touch, c.planRoot, c.planW, c.runCnt, c.planAlloc, c.winC};
  for (void* p : ps) dfree(c, p);
  c.bytes -= c.bytesParcels + c.bytesRuns;
  c.bytesParcels = c.bytesRuns = 0;
  c.capRuns = 0;
  c.runsSized = false;
  c.touchState = 0;
  c.recD[0] = c.recD[1] = nullptr;
  c.recI[0] = c.recI[1] = nullptr;
  c.imgSrc = c.imgShift = c.cellItems = c.bodyItems = c.iTmpA = c.iTmpB = c.scanScratch = c.sortHist = nullptr;
  c.kA = c.vA = c.kB = c.vB = nullptr;
  c.activeList = c.pairCnt = c.pairStart = c.pairIdx = nullptr;
  c.W = nullptr;
  c.win = nullptr;
  c.winC = nullptr;
  c.cntInt = nullptr;
  c.fv = nullptr;
  c.runStart = nullptr;
  c.runKey = nullptr;
  c.fCur = c.fPrev = nullptr;
  c.lastNodes = nullptr;
  c.touch = nullptr;
  c.planRoot = nullptr;
  c.planW = nullptr;
  c.runCnt = nullptr;
  c.planAlloc = nullptr;
  c.cap = c.capLocal = c.capImg = 0;
}

int check_params(const ibmdem_params* p) {
  if (p->nx < 4 || p->ny < 4 || p->nz < 4 || p->coupleInterval < 1 || p->Ns < 0 || !(p->dx > 0) || !(p->dy > 0) ||
      !(p->dz > 0) || !(p->dt > 0))
    return IBMDEM_EINVAL;
  // per axis: both faces periodic (0) or both solid walls (1)
  for (int d = 0; d < 3; ++d)
    if (p->bType[2 * d] != p->bType[2 * d + 1] || (p->bType[2 * d] != 0 && p->bType[2 * d] != 1))
      return IBMDEM_EUNSUPPORTED;
  long long ncell = (long long)(p->nx + 4) * (p->ny + 4) * (p->nz + 4);
  long long nint = (long long)p->nx * p->ny * p->nz;
  if (ncell >= (1ll << 31) || 3 * nint >= (1ll << 32)) return IBMDEM_EUNSUPPORTED;
  return IBMDEM_OK;
}

void init_geom(Geom& g, const ibmdem_params* p) {
  g.n[0] = p->nx;
  g.n[1] = p->ny;
  g.n[2] = p->nz;
  g.ni = p->nx + 4;
  g.nj = p->ny + 4;
  g.nk = p->nz + 4;
  g.ncell = (long long)g.ni * g.nj * g.nk;
  g.nint = (long long)p->nx * p->ny * p->nz;
  double hh[3] = {p->dx, p->dy, p->dz};
  for (int d = 0; d < 3; ++d) {
    g.h[d] = hh[d];
    g.start[d] = (1 - 1) * hh[d];
    g.end[d] = (g.n[d] - 1 + 1) * hh[d];
    g.len[d] = hh[d] * g.n[d];
    g.halfLen[d] = 0.5 * g.len[d];
    g.halfh[d] = 0.5 * hh[d];
    g.err[d] = hh[d] * 1e-20;
  }
  g.hprod = p->dx * p->dy * p->dz;
  g.unit_h = (p->dx == 1.0 && p->dy == 1.0 && p->dz == 1.0) ? 1 : 0;
  g.anyWall = 0;
  for (int d = 0; d < 3; ++d) {
    g.wall[d] = p->bType[2 * d] == 1 ? 1 : 0;
    g.anyWall |= g.wall[d];
  }
  g.dt = p->dt;
  g.rdt = 1.0 / p->dt;
  g.sdt = split_recip(p->dt);
  g.rdtLo = std::fma(-p->dt, g.rdt, 1.0) / p->dt;  // the remainder 1 - dt*rdt is exact
  g.divDt = std::isnormal(p->dt) && std::isnormal(g.rdt) && std::fabs(p->dt) < 0x1p200 && std::fabs(p->dt) > 0x1p-200
                ? 1
                : 0;
  g.dtDEM = p->dt / p->coupleInterval;
  g.rhof = p->rhof;
  g.srhof = split_recip(p->rhof);
  g.eta = eta_of(p->ResistCoeff);
  double cd = p->collisionDist * (1.0 + p->collisionBuffer);
  g.cut2 = cd * cd;
  g.knCoeff = p->knCoeff;
  g.di = p->dx;
  for (int k = 0; k < 3; ++k) g.g[k] = p->gravity[k];
  g.fdNint = FastDiv((uint32_t)g.nint);
  g.fdN0 = FastDiv((uint32_t)g.n[0]);
  g.fdN1 = FastDiv((uint32_t)g.n[1]);
  g.fdNi = FastDiv((uint32_t)g.ni);
  g.fdNj = FastDiv((uint32_t)g.nj);
}

// images the configuration needs right now (host estimate for the capacity)
long long count_images(const Geom& g, int np, const ibmdem_parcel* parts) {
  long long n = 0;
  for (int i = 0; i < np; ++i) {
    long long f = 1;
    for (int d = 0; d < 3; ++d) {
      int a = (int)std::floor((parts[i].x[d] - g.start[d]) / g.h[d]) + 1;
      int opts = 1 + ((a >= 1 && a <= kHalo) ? 1 : 0) + ((a >= g.n[d] - kHalo + 1 && a <= g.n[d]) ? 1 : 0);
      f *= opts;
    }
    n += f - 1;
  }
  return n;
}

void set_parcel_caps(Ctx& c, int np, long long nimg_est) {
  c.capLocal = std::max(np, 1);
  long long ci = nimg_est + nimg_est / 2 + 4096;
  c.capImg = (int)std::min<long long>(ci, 7ll * c.capLocal + 64);
  c.cap = c.capLocal + c.capImg;
  // the spread plan packs a parcel index with its 7-bit slot into 32 bits
  if (c.cap >= (1 << 25)) {
    c.capImg = (1 << 25) - 1 - c.capLocal;
    c.cap = c.capLocal + c.capImg;
  }
  c.capPairs = 4ll * c.capLocal + 65536;
  c.capContrib = (long long)kSlots * c.cap;
  c.capRuns = 0;  // sized from the touched nodes at the first spread plan
}

// every parcel-side device buffer with its element count, for the current caps
template <class F>
void for_each_parcel_buffer(Ctx& c, F&& f) {
  long long tmpInts = std::max<long long>(c.cap + 1, 26ll * nblocks(c.capLocal) + 1);
  long long scanInts = std::max({scan_scratch_ints(c.capRuns + 1), scan_scratch_ints(sort_hist_ints(std::max<long long>(c.cap, c.capRuns))),
                                 scan_scratch_ints(c.g.ncell + 1), scan_scratch_ints(26ll * nblocks(c.capLocal)),
                                 scan_scratch_ints(nblocks((3 * c.g.nint + 15) / 16))});
  tmpInts = std::max<long long>(tmpInts, nblocks((3 * c.g.nint + 127) / 128) + 1);
  f(c.recD[0], (size_t)ND * c.cap);
  f(c.recD[1], (size_t)ND * c.cap);
  f(c.recI[0], (size_t)NI * c.cap);
  f(c.recI[1], (size_t)NI * c.cap);
  f(c.imgSrc, (size_t)c.capImg);
  f(c.imgShift, (size_t)c.capImg);
  f(c.cellItems, (size_t)c.cap);
  f(c.bodyItems, (size_t)c.capLocal);
  f(c.iTmpA, (size_t)tmpInts);
  f(c.iTmpB, (size_t)tmpInts);
  f(c.scanScratch, (size_t)scanInts);
  f(c.sortHist, (size_t)sort_hist_ints(std::max<long long>(c.cap, c.capRuns)));
  f(c.kA, (size_t)c.cap);
  f(c.vA, (size_t)c.cap);
  f(c.kB, (size_t)c.cap);
  f(c.vB, (size_t)c.cap);
  f(c.touch, (size_t)(((3 * c.g.nint + 127) / 128) * 16));  // one bit per node, whole uint4s
  f(c.planRoot, (size_t)c.capContrib);
  f(c.planW, (size_t)c.capContrib);
  f(c.planAlloc, (size_t)1);
  f(c.activeList, (size_t)c.capLocal);
  f(c.pairCnt, (size_t)c.capLocal + 1);
  f(c.pairStart, (size_t)c.capLocal + 1);
  f(c.pairIdx, (size_t)c.capPairs);
  f(c.W, (size_t)kWStride * c.cap);
  f(c.win, (size_t)c.cap);
  f(c.winC, (size_t)c.cap);
  f(c.cntInt, (size_t)c.cap);
  f(c.fv, 3 * (size_t)c.cap);
}

// the per-touched-node arrays of the spread plan, for the current capRuns
template <class F>
void for_each_run_buffer(Ctx& c, F&& f) {
  f(c.runCnt, (size_t)c.capRuns);
  f(c.runStart, (size_t)c.capRuns + 1);
  f(c.runKey, (size_t)c.capRuns);
  f(c.fCur, (size_t)c.capRuns);
  f(c.fPrev, (size_t)c.capRuns);
  f(c.lastNodes, (size_t)c.capRuns);
}

// run capacity for `touched` nodes: room to double, never above every node
long long run_capacity(const Ctx& c, long long touched) {
  return std::min<long long>(3 * c.g.nint, std::max(2 * touched, touched + 65536));
}

int alloc_parcels(ibmdem_ctx* h, int np, long long nimg_est) {
  Ctx& c = h->c;
  free_parcel_buffers(c);
  set_parcel_caps(c, np, nimg_est);
  const size_t b0 = c.bytes;
  cudaError_t e = cudaSuccess;
  for_each_parcel_buffer(c, [&](auto& q, size_t n) {
    if (e == cudaSuccess) e = dalloc(c, q, n);
  });
  c.bytesParcels = c.bytes - b0;
  c.allocGen++;
  if (e != cudaSuccess) {
    free_parcel_buffers(c);
    return set_error(h, IBMDEM_ENOMEM, "parcel buffers: %s", cudaGetErrorString(e));
  }
  CU(cudaMemsetAsync(c.cntInt, 0, sizeof(int) * c.cap, c.stream));
  CU(cudaMemsetAsync(c.pairStart, 0, sizeof(int) * (c.capLocal + 1), c.stream));
  CU(cudaMemsetAsync(c.recD[0], 0, sizeof(double) * ND * (size_t)c.cap, c.stream));
  CU(cudaMemsetAsync(c.recI[0], 0, sizeof(int) * NI * (size_t)c.cap, c.stream));
  return IBMDEM_OK;
}

// The tangential history of the friction law for the current capacities,
// empty: no local has contacts from an earlier call, every parcel id maps to
// no local, and the next call reads side 0.
int alloc_history(ibmdem_ctx* h) {
  Ctx& c = h->c;
  free_history(c);
  const size_t b0 = c.bytes;
  cudaError_t e = cudaSuccess;
  for (int q = 0; q < 2 && e == cudaSuccess; ++q) {
    e = dalloc(c, c.histRange[q], (size_t)c.capLocal);
    if (e == cudaSuccess) e = dalloc(c, c.histGid[q], (size_t)c.capPairs);
    if (e == cudaSuccess) e = dalloc(c, c.histXi[q], 3 * (size_t)c.capPairs);
  }
  if (e == cudaSuccess) e = dalloc(c, c.pidMap, (size_t)c.capLocal);
  c.bytesHist = c.bytes - b0;
  c.allocGen++;
  if (e != cudaSuccess) {
    free_history(c);
    return set_error(h, IBMDEM_ENOMEM, "tangential history: %s", cudaGetErrorString(e));
  }
  for (int q = 0; q < 2; ++q) CU(cudaMemsetAsync(c.histRange[q], 0, sizeof(int2) * c.capLocal, c.stream));
  CU(cudaMemsetAsync(c.pidMap, 0xff, sizeof(int) * (size_t)c.capLocal, c.stream));
  CU(cudaMemsetAsync(&c.dCnt->histSide, 0, sizeof(int), c.stream));
  return IBMDEM_OK;
}

// latch device errors into a status (after a stream synchronise)
int check_device(ibmdem_ctx* h) {
  Ctx& c = h->c;
  wait_fields_read(c);  // an upload still pending finishes before the caller may reuse its arrays
  CU(cudaMemcpyAsync(c.hCnt, c.dCnt, sizeof(Counters), cudaMemcpyDeviceToHost, c.stream));
  CU(cudaStreamSynchronize(c.stream));
  if (c.planReady && c.hCnt->nRuns > 0) c.runsSeen = c.hCnt->nRuns;
  int e = c.hCnt->err;
  if (!e) return IBMDEM_OK;
  int info = c.hCnt->errInfo;
  // clear so that the context stays usable after the report
  CU(cudaMemsetAsync(&c.dCnt->err, 0, sizeof(int), c.stream));
  if (e & E_RANGE) return set_error(h, IBMDEM_ERANGE, "parcel %d left the grid and its halo", info);
  if (e & E_IMGCAP) return set_error(h, IBMDEM_ECAPACITY, "images exceed capacity %d (%d)", c.capImg, info);
  if (e & E_PAIRCAP)
    return set_error(h, IBMDEM_ECAPACITY, "contact pairs exceed capacity %lld (%d)", c.capPairs, info);
  if (e & E_PARTNER) return set_error(h, IBMDEM_ECAPACITY, "body %d has more than %d near bodies", info, c.maxPartners);
  if (e & E_WINDOW) return set_error(h, IBMDEM_EUNSUPPORTED, "parcel %d needs a 4-node delta window", info);
  if (e & E_PLANCAP) return set_error(h, IBMDEM_ECAPACITY, "spread plan exceeds capacity %lld", c.capContrib);
  if (e & E_MSIDX) return set_error(h, IBMDEM_EINVAL, "parcel %d has a body index outside 1..nMS", info);
  return set_error(h, IBMDEM_ECUDA, "device error bits 0x%x", e);
}

int launch_status(ibmdem_ctx* h) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(h, IBMDEM_ECUDA, "kernel launch failed: %s", cudaGetErrorString(e));
  return IBMDEM_OK;
}

#define CHECK_CTX()                              \
  do {                                           \
    if (!h) return IBMDEM_EINVAL;                \
    cudaError_t se_ = cudaSetDevice(h->c.device);\
    if (se_ != cudaSuccess)                      \
      return set_error(h, IBMDEM_ECUDA, "cudaSetDevice: %s", cudaGetErrorString(se_)); \
  } while (0)

#define REQUIRE(cond, msg)                                  \
  do {                                                      \
    if (!(cond)) return set_error(h, IBMDEM_ESTATE, msg);   \
  } while (0)

}  // namespace

namespace ibmdem {
static cudaEvent_t take_event(Ctx& c) {
  if (!c.evFree.empty()) {
    cudaEvent_t e = c.evFree.back();
    c.evFree.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}
static const char* const kPhaseLabels[P_COUNT] = {"interp", "spread", "weights", "plan", "cells", "pairs",
                                                  "force", "bodysum", "bodymove", "markers", "images", "reset",
                                                  "fluid_guess", "fluid_halo", "fluid_other", "fluid_poisson"};
// Every phase is an NVTX range (visible to any attached profiler, a few ns
// otherwise); with timing on it is also bracketed by CUDA events.
PhaseScope::PhaseScope(Ctx& ctx, int ph, cudaStream_t stream) : c(ctx), phase(ph), s(stream) {
  nvtxRangePushA(kPhaseLabels[ph]);
  if (!c.timing) return;
  a = take_event(c);
  b = take_event(c);
  cudaEventRecord(a, s);
}
PhaseScope::~PhaseScope() {
  nvtxRangePop();
  if (!c.timing || !a) return;
  cudaEventRecord(b, s);
  c.spans.push_back({phase, a, b});
}
static void collect_timing(Ctx& c) {
  cudaStreamSynchronize(c.stream);
  for (auto& s : c.spans) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, s.a, s.b) == cudaSuccess) {
      c.phaseMs[s.phase] += ms;
      c.phaseCount[s.phase] += 1;
    }
    c.evFree.push_back(s.a);
    c.evFree.push_back(s.b);
  }
  c.spans.clear();
}
}  // namespace ibmdem


extern "C" {

int ibmdem_timing_enable(ibmdem_ctx* h, int32_t on) {
  if (!h) return IBMDEM_EINVAL;
  h->c.timing = on != 0;
  return IBMDEM_OK;
}

const char* ibmdem_phase_name(int32_t i) { return (i >= 0 && i < P_COUNT) ? kPhaseLabels[i] : ""; }

int ibmdem_get_timing(ibmdem_ctx* h, double* ms, int64_t* counts, int32_t n, int32_t reset) {
  if (!h) return IBMDEM_EINVAL;
  Ctx& c = h->c;
  cudaSetDevice(c.device);
  collect_timing(c);
  for (int i = 0; i < n && i < P_COUNT; ++i) {
    if (ms) ms[i] = c.phaseMs[i];
    if (counts) counts[i] = c.phaseCount[i];
  }
  if (reset)
    for (int i = 0; i < P_COUNT; ++i) {
      c.phaseMs[i] = 0.0;
      c.phaseCount[i] = 0;
    }
  return P_COUNT;
}


int ibmdem_abi_version(void) { return IBMDEM_ABI_VERSION; }

const char* ibmdem_last_error(const ibmdem_ctx* h) { return h ? h->c.err.c_str() : "null context"; }

int64_t ibmdem_launch_count(const ibmdem_ctx* h) { return h ? h->c.launches : 0; }

int ibmdem_create(const ibmdem_params* p, int32_t device, ibmdem_ctx** out) {
  return create_on_stream(p, device, nullptr, out);
}

}  // extern "C"

int create_on_stream(const ibmdem_params* p, int device, cudaStream_t stream, ibmdem_ctx** out) {
  if (!p || !out) return IBMDEM_EINVAL;
  *out = nullptr;
  const int pc = check_params(p);
  if (pc) return pc;
  ibmdem_ctx* h = new (std::nothrow) ibmdem_ctx();
  if (!h) return IBMDEM_ENOMEM;
  Ctx& c = h->c;
  c.p = *p;
  c.device = device;
  c.stream = stream;
  if (cudaSetDevice(device) != cudaSuccess) {
    delete h;
    return IBMDEM_ECUDA;
  }
  retain_pool_memory(device);
  init_geom(c.g, p);

  int rc = IBMDEM_OK;
  size_t nf = (size_t)c.g.ncell;
  double** f[] = {&c.u, &c.v, &c.w, &c.u0, &c.v0, &c.w0, &c.fx, &c.fy, &c.fz};
  for (double** q : f)
    if (rc == IBMDEM_OK && dalloc(c, *q, nf) != cudaSuccess) rc = IBMDEM_ENOMEM;
  if (rc == IBMDEM_OK && dalloc(c, c.cellStart, nf + 1) != cudaSuccess) rc = IBMDEM_ENOMEM;
  if (rc == IBMDEM_OK && dalloc(c, c.cellCount, nf + 1) != cudaSuccess) rc = IBMDEM_ENOMEM;
  if (rc == IBMDEM_OK && dalloc(c, c.dCnt, 1) != cudaSuccess) rc = IBMDEM_ENOMEM;
  if (rc == IBMDEM_OK && dalloc(c, c.dTotal, 4) != cudaSuccess) rc = IBMDEM_ENOMEM;
  if (rc == IBMDEM_OK && !(c.hCnt = pinned_counters())) rc = IBMDEM_ENOMEM;
  if (rc == IBMDEM_OK) {
    for (double** q : f) cudaMemsetAsync(*q, 0, nf * sizeof(double), c.stream);
    cudaMemsetAsync(c.dCnt, 0, sizeof(Counters), c.stream);
    cudaMemsetAsync(c.cellStart, 0, sizeof(int) * (nf + 1), c.stream);
    cudaMemsetAsync(c.cellCount, 0, sizeof(int) * (nf + 1), c.stream);
    if (cudaStreamSynchronize(c.stream) != cudaSuccess) rc = IBMDEM_ECUDA;
  }
  if (rc != IBMDEM_OK) {
    ibmdem_destroy(h);
    return rc;
  }
  *out = h;
  return IBMDEM_OK;
}

extern "C" {

int ibmdem_destroy(ibmdem_ctx* h) {
  if (!h) return IBMDEM_EINVAL;
  Ctx& c = h->c;
  cudaSetDevice(c.device);
  if (c.stepBatch) ibmdem_batch_destroy(static_cast<ibmdem_batch*>(c.stepBatch));
  c.stepBatch = nullptr;
  output_release(c);
  fluid_update_release(c);
  fluid_release(c);
  poisson_release(c);
  cudaStreamSynchronize(c.stream);
  free_parcel_buffers(c);
  void* ps[] = {c.u, c.v, c.w, c.u0, c.v0, c.w0, c.fx, c.fy, c.fz, c.cellStart, c.cellCount, c.dCnt, c.dTotal, c.dBodies,
                c.bodyStart, c.bodyR2, c.partnerCnt, c.partners, c.dProbes};
  for (void* p : ps) dfree(c, p);
  // the frees are ordered on the context's stream; let them complete before
  // the stream may be destroyed by its owner
  cudaStreamSynchronize(c.stream);
  release_counters(c.hCnt);
  for (auto& sp : c.spans) {
    cudaEventDestroy(sp.a);
    cudaEventDestroy(sp.b);
  }
  for (cudaEvent_t e : c.evFree) cudaEventDestroy(e);
  if (c.fieldsRead) cudaEventDestroy(c.fieldsRead);
  if (c.upStart) cudaEventDestroy(c.upStart);
  for (cudaEvent_t e : c.compDone)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : c.upDone)
    if (e) cudaEventDestroy(e);
  if (c.upStream) cudaStreamDestroy(c.upStream);
  delete h;
  return IBMDEM_OK;
}

int ibmdem_case_bytes(const ibmdem_params* p, int32_t np, const ibmdem_parcel* parts, int32_t nMS, int64_t* bytes) {
  if (!p || !bytes || np < 0 || nMS < 0 || (np > 0 && !parts)) return IBMDEM_EINVAL;
  const int pc = check_params(p);
  if (pc) return pc;
  Ctx c;
  init_geom(c.g, p);
  const long long nf = c.g.ncell;
  long long b = 9 * nf * (long long)sizeof(double) + (nf + 1) * (long long)sizeof(int) + (long long)sizeof(Counters) +
                4 * (long long)sizeof(int);
  set_parcel_caps(c, np, count_images(c.g, np, parts));
  for_each_parcel_buffer(c, [&](auto& q, size_t n) { b += (long long)(std::max<size_t>(n, 1) * sizeof(*q)); });
  // touched nodes: about 8 per marker on a closed surface with marker spacing h
  c.capRuns = run_capacity(c, 8ll * c.cap);
  for_each_run_buffer(c, [&](auto& q, size_t n) { b += (long long)(std::max<size_t>(n, 1) * sizeof(*q)); });
  const long long nb = std::max(nMS, 1);
  b += nb * (long long)sizeof(ibmdem_multisphere) + (nb + 1) * 4 + nb * 4 + nb * 4 + nb * (long long)c.maxPartners * 4;
  *bytes = b;
  return IBMDEM_OK;
}

int ibmdem_set_stream(ibmdem_ctx* h, void* stream) {
  CHECK_CTX();
  h->c.stream = reinterpret_cast<cudaStream_t>(stream);
  return IBMDEM_OK;
}

int ibmdem_synchronize(ibmdem_ctx* h) {
  CHECK_CTX();
  int rc = launch_status(h);
  if (rc) return rc;
  return check_device(h);
}

static int ensure_plan(ibmdem_ctx* h);

static int set_fluid(ibmdem_ctx* h, const double* u, const double* v, const double* w, bool async) {
  CHECK_CTX();
  if (!u || !v || !w) return set_error(h, IBMDEM_EINVAL, "null field");
  Ctx& c = h->c;
  wait_fields_read(c);
  c.compDoneAt = -1;  // the fields change: no read-out may start from the last forcing loop's marks
  // a sparse read-out may still be writing the caller's arrays
  int ru = fluid_update_join(c);
  if (ru) return ru;
  size_t nb = sizeof(double) * (size_t)c.g.ncell;
  // With the weights of a new parcel state and no plan for them yet, the
  // spread plan (which does not read the fluid) is built on the context's
  // stream while the fields upload on a second one.
  const bool planBeside = c.weightsLocal && c.weightsGhost && !c.planReady;
  double* dst[3] = {c.u, c.v, c.w};
  double* frozen[3] = {c.u0, c.v0, c.w0};
  const double* src[3] = {u, v, w};
  if (async) {
    // Everything of the fields on a second stream, component by component:
    // the upload, then its frozen copy.  The context's stream clears the
    // forcing and builds the plan meanwhile, and the forcing loop waits for
    // each component only when it reaches it (mdf).
    if (!c.upStream) CU(cudaStreamCreateWithFlags(&c.upStream, cudaStreamNonBlocking));
    if (!c.upStart) CU(cudaEventCreateWithFlags(&c.upStart, cudaEventDisableTiming));
    for (cudaEvent_t& e : c.upDone)
      if (!e) CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    CU(cudaEventRecord(c.upStart, c.stream));
    CU(cudaStreamWaitEvent(c.upStream, c.upStart, 0));
    for (int q = 0; q < 3; ++q) {
      CU(cudaMemcpyAsync(dst[q], src[q], nb, cudaMemcpyHostToDevice, c.upStream));
      CU(cudaMemcpyAsync(frozen[q], dst[q], nb, cudaMemcpyDeviceToDevice, c.upStream));
      CU(cudaEventRecord(c.upDone[q], c.upStream));
    }
    c.uploadPending = true;
    CU(cudaMemsetAsync(c.fx, 0, nb, c.stream));
    CU(cudaMemsetAsync(c.fy, 0, nb, c.stream));
    CU(cudaMemsetAsync(c.fz, 0, nb, c.stream));
    CU(cudaMemsetAsync(&c.dCnt->nLast, 0, sizeof(int), c.stream));
    c.haveFluid = true;
    if (planBeside) return ensure_plan(h);
    return launch_status(h);
  }
  if (planBeside) {
    // The uploads go on a second stream; the context's stream clears the
    // forcing and builds the plan meanwhile, then copies each component to the
    // frozen field as soon as it has arrived (only the last copy follows the
    // last upload).
    if (!c.upStream) CU(cudaStreamCreateWithFlags(&c.upStream, cudaStreamNonBlocking));
    if (!c.upStart) CU(cudaEventCreateWithFlags(&c.upStart, cudaEventDisableTiming));
    for (cudaEvent_t& e : c.upDone)
      if (!e) CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    CU(cudaEventRecord(c.upStart, c.stream));  // after all earlier work on the fields
    CU(cudaStreamWaitEvent(c.upStream, c.upStart, 0));
    for (int q = 0; q < 3; ++q) {
      CU(cudaMemcpyAsync(dst[q], src[q], nb, cudaMemcpyHostToDevice, c.upStream));
      CU(cudaEventRecord(c.upDone[q], c.upStream));
    }
    CU(cudaMemsetAsync(c.fx, 0, nb, c.stream));
    CU(cudaMemsetAsync(c.fy, 0, nb, c.stream));
    CU(cudaMemsetAsync(c.fz, 0, nb, c.stream));
    CU(cudaMemsetAsync(&c.dCnt->nLast, 0, sizeof(int), c.stream));
    int rp = ensure_plan(h);
    // the fields are in place before any later work of the context's stream
    for (int q = 0; q < 3; ++q) {
      CU(cudaStreamWaitEvent(c.stream, c.upDone[q], 0));
      CU(cudaMemcpyAsync(frozen[q], dst[q], nb, cudaMemcpyDeviceToDevice, c.stream));
    }
    if (rp) {
      cudaStreamSynchronize(c.stream);
      return rp;
    }
  } else {
    for (int q = 0; q < 3; ++q) CU(cudaMemcpyAsync(dst[q], src[q], nb, cudaMemcpyHostToDevice, c.stream));
    for (int q = 0; q < 3; ++q) CU(cudaMemcpyAsync(frozen[q], dst[q], nb, cudaMemcpyDeviceToDevice, c.stream));
    CU(cudaMemsetAsync(c.fx, 0, nb, c.stream));
    CU(cudaMemsetAsync(c.fy, 0, nb, c.stream));
    CU(cudaMemsetAsync(c.fz, 0, nb, c.stream));
    CU(cudaMemsetAsync(&c.dCnt->nLast, 0, sizeof(int), c.stream));
  }
  c.haveFluid = true;
  // synchronous for pageable host memory semantics: the caller may reuse u,v,w
  CU(cudaStreamSynchronize(c.stream));
  return IBMDEM_OK;
}

int ibmdem_set_fluid(ibmdem_ctx* h, const double* u, const double* v, const double* w) {
  return set_fluid(h, u, v, w, false);
}

int ibmdem_set_fluid_async(ibmdem_ctx* h, const double* u, const double* v, const double* w) {
  return set_fluid(h, u, v, w, true);
}

int ibmdem_get_fluid_async(ibmdem_ctx* h, double* u, double* v, double* w, double* fx, double* fy, double* fz,
                           void* copy_stream) {
  CHECK_CTX();
  Ctx& c = h->c;
  cudaStream_t cs = reinterpret_cast<cudaStream_t>(copy_stream);
  if (cs == c.stream) return set_error(h, IBMDEM_EINVAL, "copy_stream must differ from the context's stream");
  if (!c.fieldsRead) CU(cudaEventCreateWithFlags(&c.fieldsRead, cudaEventDisableTiming));
  const size_t nb = sizeof(double) * (size_t)c.g.ncell;
  double* dst[6] = {u, v, w, fx, fy, fz};
  double* src[6] = {c.u, c.v, c.w, c.fx, c.fy, c.fz};
  if (c.compDoneAt == c.launches) {
    // right after a MDF loop: each component's velocity and forcing leave as
    // soon as that component is done, while the next ones are still computed
    for (int q = 0; q < 3; ++q) {
      CU(cudaStreamWaitEvent(cs, c.compDone[q], 0));
      if (dst[q]) CU(cudaMemcpyAsync(dst[q], src[q], nb, cudaMemcpyDeviceToHost, cs));
      if (dst[q + 3]) CU(cudaMemcpyAsync(dst[q + 3], src[q + 3], nb, cudaMemcpyDeviceToHost, cs));
    }
  } else {
    // the copies start after the work issued so far on the context's stream
    CU(cudaEventRecord(c.fieldsRead, c.stream));
    CU(cudaStreamWaitEvent(cs, c.fieldsRead, 0));
    for (int q = 0; q < 6; ++q)
      if (dst[q]) CU(cudaMemcpyAsync(dst[q], src[q], nb, cudaMemcpyDeviceToHost, cs));
  }
  // ... and the next context work that writes the fields waits for them
  CU(cudaEventRecord(c.fieldsRead, cs));
  c.fieldsReadPending = true;
  return launch_status(h);
}

int ibmdem_get_fluid(ibmdem_ctx* h, double* u, double* v, double* w, double* fx, double* fy, double* fz) {
  CHECK_CTX();
  Ctx& c = h->c;
  wait_fields_read(c);
  size_t nb = sizeof(double) * (size_t)c.g.ncell;
  double* dst[6] = {u, v, w, fx, fy, fz};
  double* src[6] = {c.u, c.v, c.w, c.fx, c.fy, c.fz};
  for (int q = 0; q < 6; ++q)
    if (dst[q]) CU(cudaMemcpyAsync(dst[q], src[q], nb, cudaMemcpyDeviceToHost, c.stream));
  return check_device(h);
}

int ibmdem_set_parcels(ibmdem_ctx* h, int32_t np, const ibmdem_parcel* parts) {
  CHECK_CTX();
  if (np < 0 || (np > 0 && !parts)) return set_error(h, IBMDEM_EINVAL, "bad parcel array");
  if (np >= (1 << 24)) return set_error(h, IBMDEM_EUNSUPPORTED, "too many parcels");
  Ctx& c = h->c;
  CU(cudaStreamSynchronize(c.stream));
  long long nimg = count_images(c.g, np, parts);
  int rc = alloc_parcels(h, np, nimg);
  if (rc) return rc;
  if (c.ktRatio > 0.0 && (rc = alloc_history(h))) return rc;
  std::vector<double> hd((size_t)ND * c.cap, 0.0);
  std::vector<int> hi((size_t)NI * c.cap, 0);
  for (int i = 0; i < np; ++i) {
    const ibmdem_parcel& p = parts[i];
    const double* src[ND];
    for (int k = 0; k < 3; ++k) {
      src[D_X + k] = &p.x[k];
      src[D_V + k] = &p.v[k];
      src[D_FCOL + k] = &p.fcol[k];
      src[D_FDRAG + k] = &p.fdrag[k];
      src[D_VGAP + k] = &p.vgap[k];
    }
    src[D_RADEFF] = &p.radeff;
    src[D_RAD] = &p.rad;
    src[D_RHO] = &p.rho;
    src[D_VOL] = &p.vol;
    src[D_M] = &p.m;
    src[D_WDRAG] = &p.wdrag;
    src[D_WSUM] = &p.wsum;
    for (int f = 0; f < ND; ++f) hd[(size_t)f * c.cap + i] = *src[f];
    hi[(size_t)I_GIDX * c.cap + i] = p.globalIdx;
    hi[(size_t)I_MSIDX * c.cap + i] = p.MSIdx;
    hi[(size_t)I_PID * c.cap + i] = i;
    int a[3];
    bool in = std::isfinite(p.x[0]) && std::isfinite(p.x[1]) && std::isfinite(p.x[2]);
    for (int d = 0; d < 3; ++d) a[d] = in ? (int)std::floor((p.x[d] - c.g.start[d]) / c.g.h[d]) + 1 : 0;
    for (int d = 0; d < 3; ++d) in = in && a[d] >= -1 && a[d] <= c.g.n[d] + 2;
    if (!in) return set_error(h, IBMDEM_ERANGE, "parcel %d at (%g,%g,%g) exceeds the region", i + 1, p.x[0], p.x[1], p.x[2]);
    hi[(size_t)I_CELL * c.cap + i] = cell_id(c.g, a[0], a[1], a[2]);
  }
  CU(cudaMemcpyAsync(c.recD[c.cur], hd.data(), sizeof(double) * hd.size(), cudaMemcpyHostToDevice, c.stream));
  CU(cudaMemcpyAsync(c.recI[c.cur], hi.data(), sizeof(int) * hi.size(), cudaMemcpyHostToDevice, c.stream));
  Counters hc{};
  hc.npLocal = hc.np = np;
  CU(cudaMemcpyAsync(c.dCnt, &hc, sizeof hc, cudaMemcpyHostToDevice, c.stream));
  // new parcels start from clean cell counts (a rebuild stopped by an error
  // may have left some behind)
  CU(cudaMemsetAsync(c.cellCount, 0, sizeof(int) * (c.g.ncell + 1), c.stream));
  CU(cudaStreamSynchronize(c.stream));
  c.haveParcels = true;
  c.listsBuilt = c.weightsLocal = c.weightsGhost = c.planReady = c.spreadValid = false;
  c.touchState = 0;
  return IBMDEM_OK;
}

int ibmdem_get_parcels(ibmdem_ctx* h, ibmdem_parcel* parts, int32_t cap, int32_t* np_out, int32_t* nlocal_out) {
  CHECK_CTX();
  Ctx& c = h->c;
  int rc = check_device(h);
  if (rc) return rc;
  int np = c.hCnt->np, nl = c.hCnt->npLocal;
  if (np_out) *np_out = np;
  if (nlocal_out) *nlocal_out = nl;
  if (!parts || np == 0) return IBMDEM_OK;
  int n = std::min(np, cap);
  std::vector<double> hd((size_t)ND * c.cap);
  std::vector<int> hi((size_t)NI * c.cap);
  CU(cudaMemcpyAsync(hd.data(), c.recD[c.cur], sizeof(double) * hd.size(), cudaMemcpyDeviceToHost, c.stream));
  CU(cudaStreamSynchronize(c.stream));
  CU(cudaMemcpyAsync(hi.data(), c.recI[c.cur], sizeof(int) * hi.size(), cudaMemcpyDeviceToHost, c.stream));
  CU(cudaStreamSynchronize(c.stream));
  // images made across a solid wall carry pType 1 (ZJS_MPI_DEM.F90:200)
  std::vector<int> shift(std::max(n - nl, 0));
  if (!shift.empty()) {
    CU(cudaMemcpyAsync(shift.data(), c.imgShift, sizeof(int) * shift.size(), cudaMemcpyDeviceToHost, c.stream));
    CU(cudaStreamSynchronize(c.stream));
  }
  for (int i = 0; i < n; ++i) {
    ibmdem_parcel& p = parts[i];
    std::memset(&p, 0, sizeof p);
    auto D = [&](int f) { return hd[(size_t)f * c.cap + i]; };
    for (int k = 0; k < 3; ++k) {
      p.x[k] = D(D_X + k);
      p.v[k] = D(D_V + k);
      p.fcol[k] = D(D_FCOL + k);
      p.fdrag[k] = D(D_FDRAG + k);
      p.vgap[k] = D(D_VGAP + k);
    }
    p.radeff = D(D_RADEFF);
    p.rad = D(D_RAD);
    p.rho = D(D_RHO);
    p.vol = D(D_VOL);
    p.m = D(D_M);
    p.wdrag = D(D_WDRAG);
    p.wsum = D(D_WSUM);
    p.globalIdx = hi[(size_t)I_GIDX * c.cap + i];
    p.MSIdx = hi[(size_t)I_MSIDX * c.cap + i];
    p.cellIdx = hi[(size_t)I_CELL * c.cap + i];
    p.localIdx = i + 1;
    p.pType = (i >= nl && ((shift[i - nl] >> kWallImgBit) & 1)) ? 1 : -1;
  }
  return IBMDEM_OK;
}

int ibmdem_set_bodies(ibmdem_ctx* h, int32_t nMS, const ibmdem_multisphere* ms) {
  CHECK_CTX();
  if (nMS < 0 || (nMS > 0 && !ms)) return set_error(h, IBMDEM_EINVAL, "bad body array");
  Ctx& c = h->c;
  CU(cudaStreamSynchronize(c.stream));
  if (nMS > c.capMS) {
    dfree(c, c.dBodies);
    dfree(c, c.bodyStart);
    dfree(c, c.bodyR2);
    dfree(c, c.partnerCnt);
    dfree(c, c.partners);
    c.dBodies = nullptr;
    c.bodyStart = nullptr;
    c.bodyR2 = nullptr;
    c.partnerCnt = c.partners = nullptr;
    CU(dalloc(c, c.dBodies, nMS));
    CU(dalloc(c, c.bodyStart, nMS + 1));
    CU(dalloc(c, c.bodyR2, nMS));
    CU(dalloc(c, c.partnerCnt, nMS));
    CU(dalloc(c, c.partners, (size_t)nMS * c.maxPartners));
    c.capMS = nMS;
    c.allocGen++;
  }
  if (nMS > 0) {
    CU(cudaMemcpyAsync(c.dBodies, ms, sizeof(ibmdem_multisphere) * nMS, cudaMemcpyHostToDevice, c.stream));
    CU(cudaStreamSynchronize(c.stream));
  }
  c.nMS = nMS;
  c.listsBuilt = false;  // body lists are built with the cell lists
  return IBMDEM_OK;
}

int ibmdem_get_bodies(ibmdem_ctx* h, ibmdem_multisphere* ms, int32_t cap, int32_t* nMS_out) {
  CHECK_CTX();
  Ctx& c = h->c;
  int rc = check_device(h);
  if (rc) return rc;
  if (nMS_out) *nMS_out = c.nMS;
  if (ms && c.nMS > 0)
    CU(cudaMemcpyAsync(ms, c.dBodies, sizeof(ibmdem_multisphere) * std::min(c.nMS, cap), cudaMemcpyDeviceToHost, c.stream));
  CU(cudaStreamSynchronize(c.stream));
  return IBMDEM_OK;
}

int ibmdem_get_cell_lists(ibmdem_ctx* h, int32_t* cell_start, int32_t* items, int64_t* ncell_out,
                          int32_t* nitems_out) {
  CHECK_CTX();
  Ctx& c = h->c;
  int rc = check_device(h);
  if (rc) return rc;
  if (ncell_out) *ncell_out = c.g.ncell;
  if (nitems_out) *nitems_out = c.hCnt->np;
  REQUIRE(c.listsBuilt, "cell lists are not built");
  if (cell_start) CU(cudaMemcpyAsync(cell_start, c.cellStart, sizeof(int) * (c.g.ncell + 1), cudaMemcpyDeviceToHost, c.stream));
  CU(cudaStreamSynchronize(c.stream));
  if (items) {
    int n = c.hCnt->np;
    CU(cudaMemcpyAsync(items, c.cellItems, sizeof(int) * n, cudaMemcpyDeviceToHost, c.stream));
    CU(cudaStreamSynchronize(c.stream));
    for (int i = 0; i < n; ++i) items[i] += 1;
  }
  return IBMDEM_OK;
}

int ibmdem_get_collision_lists(ibmdem_ctx* h, int32_t* start, int32_t* idx, int32_t* nlocal_out,
                               int32_t* npairs_out) {
  CHECK_CTX();
  Ctx& c = h->c;
  int rc = check_device(h);
  if (rc) return rc;
  REQUIRE(c.listsBuilt, "collision lists are not built");
  int nl = c.hCnt->npLocal, npairs = c.hCnt->nPairs;
  if (nlocal_out) *nlocal_out = nl;
  if (npairs_out) *npairs_out = npairs;
  if (start) CU(cudaMemcpyAsync(start, c.pairStart, sizeof(int) * (nl + 1), cudaMemcpyDeviceToHost, c.stream));
  CU(cudaStreamSynchronize(c.stream));
  if (idx) {
    CU(cudaMemcpyAsync(idx, c.pairIdx, sizeof(int) * npairs, cudaMemcpyDeviceToHost, c.stream));
    CU(cudaStreamSynchronize(c.stream));
    for (int i = 0; i < npairs; ++i) idx[i] += 1;
  }
  return IBMDEM_OK;
}

int ibmdem_get_counters(ibmdem_ctx* h, int64_t* out, int32_t n) {
  CHECK_CTX();
  Ctx& c = h->c;
  // the touched nodes and contributions are those of the plan the next spread
  // uses: build it if the weights changed since the last one
  if (c.weightsLocal && c.weightsGhost && !c.planReady) {
    int rp = ensure_plan(h);
    if (rp) return rp;
  }
  int rc = check_device(h);
  if (rc) return rc;
  int64_t v[7] = {c.hCnt->npLocal, c.hCnt->np, c.hCnt->nPairs, 0, 0, 0, c.hCnt->nContrib};
  // touched nodes per component from the run keys
  if (c.planReady && c.hCnt->nRuns > 0) {
    std::vector<uint32_t> keys(c.hCnt->nRuns);
    CU(cudaMemcpyAsync(keys.data(), c.runKey, sizeof(uint32_t) * keys.size(), cudaMemcpyDeviceToHost, c.stream));
    CU(cudaStreamSynchronize(c.stream));
    for (uint32_t k : keys) v[3 + (int)(k / (uint32_t)c.g.nint)]++;
  }
  for (int q = 0; q < n && q < 7; ++q) out[q] = v[q];
  return IBMDEM_OK;
}

// ---- reference subroutines ------------------------------------------------

static int plan(ibmdem_ctx* h);
static int size_runs(ibmdem_ctx* h);

int ibmdem_RebuildAllListOrNot(ibmdem_ctx* h) {
  CHECK_CTX();
  Ctx& c = h->c;
  REQUIRE(c.haveParcels, "no parcels");
  rebuild_cell_lists(c);
  rebuild_collision_lists(c);
  c.listsBuilt = true;
  c.weightsLocal = c.weightsGhost = c.planReady = c.spreadValid = false;
  c.touchState = 0;
  return launch_status(h);
}

int ibmdem_UpdateLocalCellWeightListDEM(ibmdem_ctx* h) {
  CHECK_CTX();
  Ctx& c = h->c;
  REQUIRE(c.listsBuilt, "lists are not built");
  launch_weights(c, true);
  c.weightsLocal = true;
  c.planReady = false;
  return launch_status(h);
}

int ibmdem_UpdateGhostCellWeightListDEM(ibmdem_ctx* h) {
  CHECK_CTX();
  Ctx& c = h->c;
  REQUIRE(c.listsBuilt, "lists are not built");
  launch_weights(c, false);
  c.weightsGhost = true;
  c.planReady = false;
  // size the spread plan's run arrays here, outside any stream capture (this
  // synchronises); the plan itself is built by the next spread, as after a
  // sub-step, so that a step leaves the host state it found
  if (c.weightsLocal && !c.runsSized) {
    int rc = size_runs(h);
    if (rc) return rc;
  }
  return launch_status(h);
}

int ibmdem_UpdateParcelInfoInGhostRegion(ibmdem_ctx* h) {
  CHECK_CTX();
  Ctx& c = h->c;
  REQUIRE(c.haveParcels, "no parcels");
  launch_img_update(c);
  return launch_status(h);
}

int ibmdem_CalculateCollisionForce(ibmdem_ctx* h) {
  CHECK_CTX();
  Ctx& c = h->c;
  REQUIRE(c.listsBuilt, "lists are not built");
  launch_collision_force(c);
  return launch_status(h);
}

int ibmdem_CalculateSolidBoundaryCollisionForce(ibmdem_ctx* h) {
  CHECK_CTX();
  Ctx& c = h->c;
  REQUIRE(c.listsBuilt, "lists are not built");
  launch_wall_force(c);
  return launch_status(h);
}

int ibmdem_set_friction(ibmdem_ctx* h, double ktRatio, double mu) {
  CHECK_CTX();
  Ctx& c = h->c;
  if (!(ktRatio >= 0.0) || !(mu >= 0.0) || !std::isfinite(ktRatio) || !std::isfinite(mu))
    return set_error(h, IBMDEM_EINVAL, "friction: ktRatio %g and mu %g must be finite and >= 0", ktRatio, mu);
  CU(cudaStreamSynchronize(c.stream));
  c.ktRatio = ktRatio;
  c.mu = mu;
  if (ktRatio > 0.0 && c.haveParcels) return alloc_history(h);
  free_history(c);
  c.allocGen++;
  return IBMDEM_OK;
}

int ibmdem_get_friction_history(ibmdem_ctx* h, int32_t* start, int32_t* gid, double* xi, int32_t* nlocal_out,
                                int32_t* n_out) {
  CHECK_CTX();
  Ctx& c = h->c;
  int rc = check_device(h);
  if (rc) return rc;
  const int nl = c.pidMap ? c.hCnt->npLocal : 0;
  if (nlocal_out) *nlocal_out = nl;
  if (n_out) *n_out = 0;
  if (nl == 0) {
    if (start) start[0] = 0;
    return IBMDEM_OK;
  }
  const int side = c.hCnt->histSide;  // the side the last call wrote
  std::vector<int2> r(nl);
  CU(cudaMemcpyAsync(r.data(), c.histRange[side], sizeof(int2) * nl, cudaMemcpyDeviceToHost, c.stream));
  CU(cudaStreamSynchronize(c.stream));
  const int first = r[0].x, total = r[nl - 1].y - first;
  if (n_out) *n_out = total;
  if (start) {
    for (int i = 0; i < nl; ++i) start[i] = r[i].x - first;
    start[nl] = total;
  }
  if (gid && total > 0)
    CU(cudaMemcpyAsync(gid, c.histGid[side] + first, sizeof(int) * total, cudaMemcpyDeviceToHost, c.stream));
  if (xi && total > 0)
    CU(cudaMemcpyAsync(xi, c.histXi[side] + 3 * (size_t)first, sizeof(double) * 3 * total, cudaMemcpyDeviceToHost,
                       c.stream));
  CU(cudaStreamSynchronize(c.stream));
  return IBMDEM_OK;
}

int ibmdem_set_wall_probes(ibmdem_ctx* h, int32_t n, const ibmdem_wall_probe* probes) {
  CHECK_CTX();
  Ctx& c = h->c;
  if (n < 0 || n > IBMDEM_MAX_WALL_PROBES || (n > 0 && !probes))
    return set_error(h, IBMDEM_EINVAL, "%d wall probes (at most %d)", n, IBMDEM_MAX_WALL_PROBES);
  std::vector<ibmdem_wall_probe> hp(probes, probes + n);
  for (int q = 0; q < n; ++q) {
    if (hp[q].face < 1 || hp[q].face > 6 || !c.g.wall[(hp[q].face - 1) / 2])
      return set_error(h, IBMDEM_EINVAL, "wall probe %d: face %d is not a solid wall", q, hp[q].face);
    hp[q].force[0] = hp[q].force[1] = hp[q].force[2] = 0.0;
  }
  if (!c.dProbes && dalloc(c, c.dProbes, IBMDEM_MAX_WALL_PROBES) != cudaSuccess)
    return set_error(h, IBMDEM_ENOMEM, "wall probes");
  if (n) CU(cudaMemcpyAsync(c.dProbes, hp.data(), sizeof(ibmdem_wall_probe) * n, cudaMemcpyHostToDevice, c.stream));
  CU(cudaStreamSynchronize(c.stream));
  c.nProbe = n;
  return launch_status(h);
}

int ibmdem_get_wall_probes(ibmdem_ctx* h, ibmdem_wall_probe* probes, int32_t cap, int32_t* n_out) {
  CHECK_CTX();
  Ctx& c = h->c;
  if (n_out) *n_out = c.nProbe;
  const int n = std::min<int>(c.nProbe, std::max(cap, 0));
  if (probes && n > 0) {
    CU(cudaMemcpyAsync(probes, c.dProbes, sizeof(ibmdem_wall_probe) * n, cudaMemcpyDeviceToHost, c.stream));
    CU(cudaStreamSynchronize(c.stream));
  }
  return check_device(h);
}

int ibmdem_UpdateFluidVelocityOnLagrangianPoints(ibmdem_ctx* h) {
  CHECK_CTX();
  Ctx& c = h->c;
  REQUIRE(c.weightsLocal, "local weights are not computed");
  REQUIRE(c.haveFluid, "no fluid field");
  wait_fields_read(c);  // an ibmdem_set_fluid_async upload lands before the fields are read
  launch_interp(c, -1);
  return launch_status(h);
}

// Allocate the run arrays for the nodes the current weights touch (counted on
// the device; synchronises), with room to double.  Done once per parcel set,
// before the first spread plan, outside any stream capture.
static int size_runs(ibmdem_ctx* h) {
  Ctx& c = h->c;
  const long long touched = count_touched_nodes(c);
  if (touched < 0) return set_error(h, IBMDEM_ECUDA, "counting touched nodes failed");
  for_each_run_buffer(c, [&](auto& q, size_t) {
    dfree(c, q);
    q = nullptr;
  });
  c.bytes -= c.bytesRuns;
  c.capRuns = run_capacity(c, touched);
  c.runsSeen = touched;
  const size_t b0 = c.bytes;
  cudaError_t e = cudaSuccess;
  for_each_run_buffer(c, [&](auto& q, size_t n) {
    if (e == cudaSuccess) e = dalloc(c, q, n);
  });
  c.bytesRuns = c.bytes - b0;
  c.allocGen++;
  if (e != cudaSuccess) return set_error(h, IBMDEM_ENOMEM, "spread-plan runs: %s", cudaGetErrorString(e));
  c.runsSized = true;
  return IBMDEM_OK;
}

static int plan(ibmdem_ctx* h) {
  Ctx& c = h->c;
  if (!c.runsSized) {
    int rc = size_runs(h);
    if (rc) return rc;
  }
  build_spread_plan(c);
  return IBMDEM_OK;
}

static int ensure_plan(ibmdem_ctx* h) {
  Ctx& c = h->c;
  REQUIRE(c.weightsLocal && c.weightsGhost, "weights are not computed");
  if (!c.planReady) {
    PhaseScope t(c, P_PLAN);
    return plan(h);
  }
  return IBMDEM_OK;
}

int ibmdem_UpdateMomentumSourceTerm(ibmdem_ctx* h) {
  CHECK_CTX();
  Ctx& c = h->c;
  wait_fields_read(c);
  int rc = ensure_plan(h);
  if (rc) return rc;
  REQUIRE(c.spreadValid, "spreading needs MultiDirectForcing's reset after the weights change");
  launch_spread(c, false, -1);
  return launch_status(h);
}

int ibmdem_VelocityPostGuess(ibmdem_ctx* h) {
  CHECK_CTX();
  Ctx& c = h->c;
  wait_fields_read(c);
  REQUIRE(c.planReady && c.spreadValid, "no spread to apply");
  launch_post_guess(c);
  return launch_status(h);
}

int ibmdem_AssembleLocalForceMS(ibmdem_ctx* h) {
  CHECK_CTX();
  Ctx& c = h->c;
  REQUIRE(c.listsBuilt, "body lists are not built");
  launch_body_sums(c);
  return launch_status(h);
}

int ibmdem_EvolutionMS(ibmdem_ctx* h) {
  CHECK_CTX();
  launch_evolution(h->c);
  return launch_status(h);
}

int ibmdem_ResetVelocityAndPositionLagrangianPoints(ibmdem_ctx* h) {
  CHECK_CTX();
  REQUIRE(h->c.haveParcels, "no parcels");
  launch_marker_update(h->c, true, false);
  return launch_status(h);
}

int ibmdem_AdjustParcelPosition(ibmdem_ctx* h) {
  CHECK_CTX();
  REQUIRE(h->c.haveParcels, "no parcels");
  launch_marker_update(h->c, false, true);
  return launch_status(h);
}

// ---- drivers -----------------------------------------------------------------

int ibmdem_InitializationDEM(ibmdem_ctx* h) {
  int rc = ibmdem_RebuildAllListOrNot(h);
  if (!rc) rc = ibmdem_UpdateLocalCellWeightListDEM(h);
  if (!rc) rc = ibmdem_UpdateParcelInfoInGhostRegion(h);
  if (!rc) rc = ibmdem_UpdateGhostCellWeightListDEM(h);
  return rc;
}

// The forcing loop's set-up: the plan for the current weights and the reset.
// *first gets the first iteration's flags for launch_interp / launch_spread.
static int mdf_begin(ibmdem_ctx* h, bool frozen, int* first) {
  Ctx& c = h->c;
  // The plan for new weights does not read the fluid, but it is built here, in
  // order: beside the forcing loop on a second stream it took the loop's SMs
  // (the fill is issue-bound, the loop FP64-bound at high occupancy) and the
  // step measured 5% slower.
  int rc = ensure_plan(h);
  if (rc) return rc;
  // with at least one iteration the first one takes the reset's zeros itself
  // and only the nodes the last spread wrote outside the new plan are reset
  const bool firstFlags = c.p.Ns > 0;
  {
    PhaseScope t(c, P_RESET);
    if (firstFlags)
      launch_mdf_stale(c, frozen);
    else
      launch_mdf_reset(c, frozen);
  }
  *first = 1 | (frozen ? 2 : 0);
  return IBMDEM_OK;
}

// After the forcing loop: the images take their sources' final fdrag (the
// spread gathers the roots' fdrag*vol, never the images'), and the nodes the
// last spread wrote are kept for the next reset.
static void mdf_end(Ctx& c) {
  {
    PhaseScope t(c, P_IMAGES);
    launch_img_update(c);
  }
  {
    PhaseScope t(c, P_RESET);
    record_written_nodes(c);
  }
}

static int mdf(ibmdem_ctx* h, bool frozen) {
  Ctx& c = h->c;
  REQUIRE(c.haveFluid, "no fluid field");
  const bool perCompUpload = !frozen && c.uploadPending;  // ibmdem_set_fluid_async still uploading
  wait_fields_read(c, !perCompUpload);
  int first = 0;
  int rc = mdf_begin(h, frozen, &first);
  if (rc) return rc;
  // The three velocity components never meet inside the MDF loop (fluid.F90:
  // 265-285): a marker's component interpolates from that component of the
  // field, and the spread and the post-guess of a node write that component
  // only.  For a caller that reads the fields right after (MultiDirectForcing
  // in a coupled step) the loop runs component by component, so that the
  // read-out of u and fx can start once the first component is done
  // (ibmdem_get_fluid_async); the frozen-fluid step keeps the three
  // components in one launch, which is 3% faster on the device.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(c.stream, &cap);
  const bool byComp = !frozen && cap == cudaStreamCaptureStatusNone;
  if (!byComp) wait_fields_read(c);
  for (int comp = byComp ? 0 : -1; comp < (byComp ? 3 : 0); ++comp) {
    if (byComp && perCompUpload) cudaStreamWaitEvent(c.stream, c.upDone[comp], 0);
    for (int it = 0; it < c.p.Ns; ++it) {
      {
        PhaseScope t(c, P_INTERP);
        launch_interp(c, comp, it == 0 ? first : 0);
      }
      {
        PhaseScope t(c, P_SPREAD);
        launch_spread(c, true, comp, it == 0 ? first : 0);
      }
    }
    if (byComp) {
      if (!c.compDone[comp]) cudaEventCreateWithFlags(&c.compDone[comp], cudaEventDisableTiming);
      cudaEventRecord(c.compDone[comp], c.stream);
    }
  }
  mdf_end(c);
  if (perCompUpload) c.uploadPending = false;  // the stream has waited for the last component
  c.compDoneAt = byComp ? c.launches : -1;
  return launch_status(h);
}

}  // extern "C"

// A frozen-fluid step whose forcing loop a batch runs for all its members in
// shared launches (batch.cu): the part before the loop, and the part after it.
int step_before_forcing(ibmdem_ctx* h) {
  CHECK_CTX();
  Ctx& c = h->c;
  REQUIRE(c.haveFluid, "no fluid field");
  REQUIRE(c.p.Ns > 0, "no forcing iterations");
  wait_fields_read(c);
  int first = 0;
  int rc = mdf_begin(h, true, &first);
  if (rc) return rc;
  return launch_status(h);
}

int step_after_forcing(ibmdem_ctx* h) {
  CHECK_CTX();
  Ctx& c = h->c;
  mdf_end(c);
  c.compDoneAt = -1;
  int rc = launch_status(h);
  if (rc) return rc;
  return ibmdem_CloudEvolutionMS(h);
}

extern "C" {

int ibmdem_MultiDirectForcing(ibmdem_ctx* h) {
  CHECK_CTX();
  return mdf(h, false);
}

}  // extern "C"

// CloudEvolutionStepMS whose AssembleLocalForceMS forms the sums `sums` only
// (launch_body_sums); ibmdem_CloudEvolutionStepMS forms all of them.
static int cloud_step(ibmdem_ctx* h, int sums) {
  Ctx& c = h->c;
  REQUIRE(c.listsBuilt && c.weightsLocal && c.weightsGhost, "lists and weights are not built");
  {
    PhaseScope t(c, P_FORCE);
    launch_collision_force(c);
    launch_wall_force(c);
  }
  { PhaseScope t(c, P_BODYSUM); launch_body_sums(c, sums); }
  { PhaseScope t(c, P_BODYMOVE); launch_evolution(c); }
  { PhaseScope t(c, P_MARKERS); launch_marker_update(c, true, true); }
  { PhaseScope t(c, P_IMAGES); launch_img_update(c); }
  { PhaseScope t(c, P_CELLS); rebuild_cell_lists(c); }
  { PhaseScope t(c, P_PAIRS); rebuild_collision_lists(c); }
  { PhaseScope t(c, P_WEIGHTS); launch_weights(c, true); }
  { PhaseScope t(c, P_IMAGES); launch_img_update(c); }
  { PhaseScope t(c, P_WEIGHTS); launch_weights(c, false); }
  // the spread plan follows the new weights when a spread next needs it: of
  // coupleInterval sub-steps only the last one's plan is ever used
  c.listsBuilt = c.weightsLocal = c.weightsGhost = true;
  c.planReady = c.spreadValid = false;
  return launch_status(h);
}

extern "C" {

int ibmdem_CloudEvolutionStepMS(ibmdem_ctx* h) {
  CHECK_CTX();
  return cloud_step(h, SUMS_ALL);
}

// Each AssembleLocalForceMS of the reference forms all twelve body sums, but
// within CloudEvolutionMS (couplesolverCylinder.F90:189-217) only some of
// them are read before the next call overwrites them: the first call's fdrag
// and fmom (for fhydro, fmomHydro), each sub-step's fcol and fmomCol (for
// EvolutionMS).  The fdrag and fmom the caller sees at the end are those of
// the last call, whose markers sit where the first call's did when there is
// one sub-step (the sums are then the first call's, bit for bit) and have
// moved when there are more.  So the first call forms fdrag and fmom, the
// sub-steps fcol and fmomCol, and the last of several sub-steps all twelve.
int ibmdem_CloudEvolutionMS(ibmdem_ctx* h) {
  CHECK_CTX();
  Ctx& c = h->c;
  REQUIRE(c.listsBuilt, "lists are not built");
  { PhaseScope t(c, P_BODYMOVE); launch_cloud_pre(c); }
  { PhaseScope t(c, P_BODYSUM); launch_body_sums(c, SUMS_HYDRO); }
  { PhaseScope t(c, P_BODYMOVE); launch_cloud_post(c); }
  const int K = c.p.coupleInterval;
  for (int s = 0; s < K; ++s) {
    int rc = cloud_step(h, K > 1 && s == K - 1 ? SUMS_ALL : SUMS_COL);
    if (rc) return rc;
  }
  return launch_status(h);
}

int ibmdem_set_step_graphs(ibmdem_ctx* h, int32_t on) {
  CHECK_CTX();
  if (on != 0 && on != 1) return set_error(h, IBMDEM_EINVAL, "step graphs: 0 or 1");
  h->c.stepGraphs = on != 0;
  return IBMDEM_OK;
}

int ibmdem_step(ibmdem_ctx* h, int32_t nsteps) {
  CHECK_CTX();
  Ctx& c = h->c;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(c.stream, &cap);
  if (nsteps > 0 && c.stepGraphs && !c.timing && cap == cudaStreamCaptureStatusNone) {
    // the steps as replays of one captured graph (a batch of this case alone):
    // the same kernels, one launch per step instead of some eighty; a step
    // captured inside someone else's capture, or with phase timing on, takes
    // the stream path below
    ibmdem_batch* b = static_cast<ibmdem_batch*>(c.stepBatch);
    if (!b) {
      int rc = ibmdem_batch_create(c.device, &b);
      if (rc) return set_error(h, rc, "step graph: no batch");
      rc = ibmdem_batch_add(b, h);
      if (!rc) rc = ibmdem_batch_set_lanes(b, 1);
      if (rc) {
        ibmdem_batch_destroy(b);
        return set_error(h, rc, "step graph: batch set-up failed");
      }
      c.stepBatch = b;
    }
    const int rc = ibmdem_batch_step(b, nsteps);
    if (rc) return set_error(h, rc, "step graph: %s", ibmdem_batch_last_error(b));
    return launch_status(h);
  }
  for (int s = 0; s < nsteps; ++s) {
    int rc = mdf(h, true);
    if (rc) return rc;
    rc = ibmdem_CloudEvolutionMS(h);
    if (rc) return rc;
  }
  return IBMDEM_OK;
}

// For callers that must not allocate inside their time loop (device memory
// committed to the fluid solver's own arrays, or other streams kept busy that a
// cudaMalloc/cudaFree would synchronise): the weights go to a fixed static
// device array, so nothing is allocated here, and n is capped by its size.
int ibmdem_interpolate_velocity_noalloc(ibmdem_ctx* h, int32_t n, const double* x, double* ulp) {
  CHECK_CTX();
  Ctx& c = h->c;
  if (n < 0) return set_error(h, IBMDEM_EINVAL, "negative point count %d", n);
  if (n > IBMDEM_PROBE_MAX_POINTS)
    return set_error(h, IBMDEM_ERANGE,
                     "%d points exceed the %d that ibmdem_interpolate_velocity_noalloc holds in its static array", n,
                     IBMDEM_PROBE_MAX_POINTS);
  if (n > 0 && (!x || !ulp)) return set_error(h, IBMDEM_EINVAL, "null point or result array");
  REQUIRE(c.haveFluid, "no fluid field");
  wait_fields_read(c);  // an ibmdem_set_fluid_async upload lands before the fields are read
  int bad = -1;
  const cudaError_t e = interpolate_points_noalloc(c, n, x, ulp, &bad);
  if (e != cudaSuccess)
    return set_error(h, IBMDEM_ECUDA, "ibmdem_interpolate_velocity_noalloc: %s", cudaGetErrorString(e));
  if (bad >= 0)
    return set_error(h, IBMDEM_ERANGE, "point %d lies outside the box [0,%g) x [0,%g) x [0,%g)", bad, c.g.len[0],
                     c.g.len[1], c.g.len[2]);
  return IBMDEM_OK;
}

}  // extern "C"
