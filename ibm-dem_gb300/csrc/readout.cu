// readout.cu — the coupled caller's field read-out, sparse.
//
// After MultiDirectForcing the fields differ from what ibmdem_set_fluid loaded
// only at the nodes the spread touched (and at their halo images): u, v, w
// took the post-guess update there, and fx, fy, fz are zero everywhere else.
// A caller that keeps its own copy of the fields -- the Fortran fluid solver
// passes its arrays in and wants them back -- therefore needs only (node, u, f)
// for the touched nodes: about 20 bytes per node instead of six whole fields.
// A kernel packs them into a buffer of their own, the copy runs on the caller's
// copy stream, and a host thread writes them into the caller's arrays with the
// halo images (periodic copies, or across a wall the negated mirror with a zero
// wall-normal component, as the spread writes them on the device) and clears
// fx, fy, fz at the nodes the previous read-out wrote.
#include <algorithm>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace ibmdem {

struct FluidUpdate {
  uint32_t* dKey = nullptr;  // [cap] touched node keys
  double* dVal = nullptr;    // [2*cap] (u, f) per node
  int* dCount = nullptr;
  long long cap = 0;
  uint32_t* hKey = nullptr;  // pinned; this read-out's keys
  uint32_t* hPrev = nullptr;  // pinned; the previous read-out's keys (nPrev)
  long long nPrev = 0;
  double* hVal = nullptr;
  int* hCount = nullptr;
  long long hcap = 0;
  cudaEvent_t packed = nullptr, counted = nullptr, copied = nullptr;
  std::thread worker;
  bool pending = false;
  int status = IBMDEM_OK;
  long long lastBytes = 0;
};

namespace {

// stream-ordered device memory, as the context's other buffers
template <typename T>
cudaError_t ualloc(Ctx& c, T*& p, size_t n) {
  p = nullptr;
  const size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
  const cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&p), bytes, c.stream);
  if (e == cudaSuccess) c.bytes += bytes;
  return e;
}
void ufree(Ctx& c, void* p) {
  if (p) cudaFreeAsync(p, c.stream);
}

__global__ void k_pack_touched(Geom g, const Counters* cnt, const uint32_t* __restrict__ runKey, const double* u,
                               const double* v, const double* w, const double* fx, const double* fy, const double* fz,
                               uint32_t* key, double* val, int* count) {
  const long long n = cnt->nRuns;
  if (blockIdx.x == 0 && threadIdx.x == 0) *count = (int)n;
  for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x) {
    const uint32_t kk = runKey[r];
    const uint32_t c = g.fdNint.div(kk);
    const uint32_t node = kk - c * (uint32_t)g.nint;
    const uint32_t row = g.fdN0.div(node);
    const uint32_t kz = g.fdN1.div(row);
    const int i = (int)(node - row * (uint32_t)g.n[0]) + 1;
    const int j = (int)(row - kz * (uint32_t)g.n[1]) + 1;
    const int k = (int)kz + 1;
    const long long off = field_off(g, i, j, k);
    const double* U = c == 0 ? u : (c == 1 ? v : w);
    const double* F = c == 0 ? fx : (c == 1 ? fy : fz);
    key[r] = kk;
    val[2 * r] = U[off];
    val[2 * r + 1] = F[off];
  }
}

struct HostGeom {
  int n[3], ni, nj, wall[3];
  long long nint;
  FastDiv fdNint, fdN0, fdN1;  // the multiply-shift divisions of the device decode
  long long off(int i, int j, int k) const { return ((long long)(k + 1) * nj + (j + 1)) * ni + (i + 1); }
  void coords(uint32_t key, int& comp, int& i, int& j, int& k) const {
    const uint32_t c = fdNint.div(key);
    const uint32_t node = key - c * (uint32_t)nint;
    const uint32_t row = fdN0.div(node);
    const uint32_t kz = fdN1.div(row);
    comp = (int)c;
    i = (int)(node - row * (uint32_t)n[0]) + 1;
    j = (int)(row - kz * (uint32_t)n[1]) + 1;
    k = (int)kz + 1;
  }
};

// the node's value where the halo refill and Boundary() put it (the rules of
// the device's post-guess write)
void put_images(double* F, const HostGeom& g, int comp, int i, int j, int k, double val) {
  int pos[3][2], neg[3][2], cnt[3];
  const int id[3] = {i, j, k};
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
        double x = (neg[0][a] ^ neg[1][b] ^ neg[2][c]) ? -val : val;
        if (g.wall[comp] && (p[comp] <= 1 || p[comp] >= nc + 1)) x = 0.0;
        F[g.off(p[0], p[1], p[2])] = x;
      }
}

template <class Fn>
void parallel_for(long long n, Fn fn) {
  const int nt = (int)std::max(1ll, std::min<long long>((n + 65535) / 65536,
                                                        std::max(1u, std::min(16u, std::thread::hardware_concurrency()))));
  if (nt == 1) {
    fn(0ll, n);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t) {
    const long long a = n * t / nt, b = n * (t + 1) / nt;
    th.emplace_back([=] { fn(a, b); });
  }
  for (auto& x : th) x.join();
}

}  // namespace

void fluid_update_release(Ctx& c) {
  FluidUpdate* q = c.upd;
  if (!q) return;
  if (q->worker.joinable()) q->worker.join();
  ufree(c, q->dKey);
  ufree(c, q->dVal);
  ufree(c, q->dCount);
  if (q->hKey) cudaFreeHost(q->hKey);
  if (q->hPrev) cudaFreeHost(q->hPrev);
  if (q->hVal) cudaFreeHost(q->hVal);
  if (q->hCount) cudaFreeHost(q->hCount);
  if (q->packed) cudaEventDestroy(q->packed);
  if (q->counted) cudaEventDestroy(q->counted);
  if (q->copied) cudaEventDestroy(q->copied);
  delete q;
  c.upd = nullptr;
}

int fluid_update_join(Ctx& c) {
  FluidUpdate* q = c.upd;
  if (!q || !q->pending) return IBMDEM_OK;
  if (q->worker.joinable()) q->worker.join();
  q->pending = false;
  return q->status;
}

}  // namespace ibmdem

using namespace ibmdem;

extern "C" {

int ibmdem_update_fluid_wait(ibmdem_ctx* h) {
  if (!h) return IBMDEM_EINVAL;
  return fluid_update_join(h->c);
}

int ibmdem_update_fluid_bytes(const ibmdem_ctx* h, int64_t* bytes) {
  if (!h || !bytes) return IBMDEM_EINVAL;
  *bytes = h->c.upd ? h->c.upd->lastBytes : 0;
  return IBMDEM_OK;
}

int ibmdem_update_fluid_async(ibmdem_ctx* h, double* u, double* v, double* w, double* fx, double* fy, double* fz,
                              void* copy_stream) {
  if (!h) return IBMDEM_EINVAL;
  Ctx& c = h->c;
  if (!u || !v || !w || !fx || !fy || !fz) {
    c.err = "ibmdem_update_fluid_async: null array";
    return IBMDEM_EINVAL;
  }
  cudaStream_t cs = reinterpret_cast<cudaStream_t>(copy_stream);
  if (cs == c.stream) {
    c.err = "ibmdem_update_fluid_async: copy_stream must differ from the context's stream";
    return IBMDEM_EINVAL;
  }
  int rc = fluid_update_join(c);
  if (rc) return rc;
  if (!c.haveFluid) {
    c.err = "ibmdem_update_fluid_async: no fluid field";
    return IBMDEM_ESTATE;
  }
  if (cudaSetDevice(c.device) != cudaSuccess) return IBMDEM_ECUDA;
  if (!c.upd) c.upd = new FluidUpdate();
  FluidUpdate* q = c.upd;
  auto fail = [&](const char* what, cudaError_t e) {
    c.err = std::string("ibmdem_update_fluid_async: ") + what + ": " + cudaGetErrorString(e);
    return IBMDEM_ECUDA;
  };
  cudaError_t e = cudaSuccess;
  const long long need = std::max<long long>(c.capRuns, 1);
  if (q->cap < need) {
    ufree(c, q->dKey);
    ufree(c, q->dVal);
    q->dKey = nullptr;
    q->dVal = nullptr;
    q->cap = 0;
    if ((e = ualloc(c, q->dKey, (size_t)need)) != cudaSuccess) return fail("device buffer", e);
    if ((e = ualloc(c, q->dVal, (size_t)(2 * need))) != cudaSuccess) return fail("device buffer", e);
    q->cap = need;
  }
  if (!q->dCount && (e = ualloc(c, q->dCount, 1)) != cudaSuccess) return fail("device buffer", e);
  if (q->hcap < need) {
    // the previous keys move into the larger buffer
    uint32_t* prev = nullptr;
    if ((e = cudaMallocHost(&prev, sizeof(uint32_t) * need)) != cudaSuccess) return fail("pinned buffer", e);
    if (q->nPrev) std::memcpy(prev, q->hPrev, sizeof(uint32_t) * q->nPrev);
    if (q->hKey) cudaFreeHost(q->hKey);
    if (q->hPrev) cudaFreeHost(q->hPrev);
    if (q->hVal) cudaFreeHost(q->hVal);
    q->hKey = nullptr;
    q->hVal = nullptr;
    q->hPrev = prev;
    q->hcap = 0;
    if ((e = cudaMallocHost(&q->hKey, sizeof(uint32_t) * need)) != cudaSuccess) return fail("pinned buffer", e);
    if ((e = cudaMallocHost(&q->hVal, sizeof(double) * 2 * need)) != cudaSuccess) return fail("pinned buffer", e);
    q->hcap = need;
  }
  if (!q->hCount && (e = cudaMallocHost(&q->hCount, sizeof(int))) != cudaSuccess) return fail("pinned count", e);
  for (cudaEvent_t* ev : {&q->packed, &q->counted, &q->copied})
    if (!*ev && (e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming)) != cudaSuccess) return fail("event", e);
  // the touched nodes of the last spread and their values, after the work issued so far
  if (c.runKey && c.runsSized) {
    k_pack_touched<<<gs_blocks(c.capRuns), kBlock, 0, c.stream>>>(c.g, c.dCnt, c.runKey, c.u, c.v, c.w, c.fx, c.fy,
                                                                   c.fz, q->dKey, q->dVal, q->dCount);
    c.launches++;
  } else {
    cudaMemsetAsync(q->dCount, 0, sizeof(int), c.stream);
  }
  cudaEventRecord(q->packed, c.stream);
  cudaStreamWaitEvent(cs, q->packed, 0);
  cudaMemcpyAsync(q->hCount, q->dCount, sizeof(int), cudaMemcpyDeviceToHost, cs);
  cudaEventRecord(q->counted, cs);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail("launch", e);
  HostGeom g;
  for (int d = 0; d < 3; ++d) {
    g.n[d] = c.g.n[d];
    g.wall[d] = c.g.wall[d];
  }
  g.ni = c.g.ni;
  g.nj = c.g.nj;
  g.nint = c.g.nint;
  g.fdNint = c.g.fdNint;
  g.fdN0 = c.g.fdN0;
  g.fdN1 = c.g.fdN1;
  const int dev = c.device;
  q->pending = true;
  q->status = IBMDEM_OK;
  q->worker = std::thread([q, g, cs, dev, u, v, w, fx, fy, fz] {
    cudaSetDevice(dev);
    if (cudaEventSynchronize(q->counted) != cudaSuccess) {
      q->status = IBMDEM_ECUDA;
      return;
    }
    const long long n = std::min<long long>(*q->hCount, q->hcap);
    if (n > 0) {
      cudaMemcpyAsync(q->hKey, q->dKey, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, cs);
      cudaMemcpyAsync(q->hVal, q->dVal, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, cs);
      cudaEventRecord(q->copied, cs);
      if (cudaEventSynchronize(q->copied) != cudaSuccess) {
        q->status = IBMDEM_ECUDA;
        return;
      }
    }
    q->lastBytes = (long long)sizeof(int) + n * (long long)(sizeof(uint32_t) + 2 * sizeof(double));
    double* U[3] = {u, v, w};
    double* F[3] = {fx, fy, fz};
    const uint32_t* key = q->hKey;
    const uint32_t* prev = q->hPrev;
    const long long np = q->nPrev;
    const double* val = q->hVal;
    // one pass over the key space in parallel slices: the forcing the arrays
    // hold from the previous read-out is zeroed, except at the nodes touched
    // now, which take their u (with its halo images) and f; both key lists are
    // sorted, so each slice walks both in step
    const long long span = 3ll * g.nint;
    parallel_for(std::max(n, np), [&](long long a, long long b) {
      const long long total = std::max(n, np);
      const uint32_t lo = (uint32_t)(span * a / total), hi = (uint32_t)(span * b / total);
      long long r = std::lower_bound(key, key + n, lo) - key;
      long long s = std::lower_bound(prev, prev + np, lo) - prev;
      const long long r1 = std::lower_bound(key, key + n, hi) - key;
      const long long s1 = std::lower_bound(prev, prev + np, hi) - prev;
      int comp, i, j, k;
      while (r < r1 || s < s1) {
        if (s < s1 && (r >= r1 || prev[s] < key[r])) {
          g.coords(prev[s++], comp, i, j, k);
          F[comp][g.off(i, j, k)] = 0.0;
          continue;
        }
        if (s < s1 && prev[s] == key[r]) ++s;
        g.coords(key[r], comp, i, j, k);
        put_images(U[comp], g, comp, i, j, k, val[2 * r]);
        F[comp][g.off(i, j, k)] = val[2 * r + 1];
        ++r;
      }
    });
    std::swap(q->hKey, q->hPrev);
    q->nPrev = n;
  });
  return IBMDEM_OK;
}

}  // extern "C"
