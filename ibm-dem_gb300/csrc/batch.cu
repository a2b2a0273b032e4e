// batch.cu — many independent cases on one device: a batch advanced by one
// CUDA graph launch per step, and a request server that admits cases by device
// memory budget and overlaps them.
//
// Batch.  One frozen-fluid step of every member case (ibmdem_step) is captured
// into a single CUDA graph.  The cases are dealt onto `lanes` concurrent chains,
// largest first, each to the chain with the least work so far, so a graph
// launch advances every case by one step while the kernels of cases on
// different chains run side by side.  Each case keeps its own device state and
// its own kernels; only the issue order changes, so a case's results are the
// same in a batch as alone.  The number of chains is a tuning knob
// (ibmdem_batch_autotune times a few and keeps the fastest): many chains give
// small cases room to overlap, few chains keep large cases from contending.
// Optionally (ibmdem_batch_set_fused) the forcing loop -- two thirds of a step's
// work -- runs for all members at once: the chains build every member's plan
// and reset, join, one interpolation and one spread launch per iteration cover
// all members (each block looks its member up in a descriptor table and runs
// the per-case block code on that member's state), and the chains fork again
// for the images and CloudEvolutionMS.  The autotuner also decides between the
// two and picks the interpolation's block size.
//
// Server.  Requests wait in a queue and are admitted, in arrival order or
// least work first (ibmdem_server_set_policy), while the summed device
// footprint of the running cases (ibmdem_case_bytes) stays within the budget
// and fewer than max_active run.  An admitted case gets its
// own stream, its step captured once as a graph, and all of its steps queued
// at admission; the device interleaves the running cases.  A case whose last
// step has completed is read back and its memory returned to the pool in
// stream order, so the next request is admitted without stalling the others.
#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <new>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

using namespace ibmdem;

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

void fmt_err(std::string& dst, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  dst = buf;
}

// work estimate of one case step: parcel capacity (markers and their images)
// plus the grid it sweeps
double case_work(const Ctx& c) { return (double)c.cap * 100.0 + (double)c.g.ncell; }

// The host state a captured step depends on: buffer generation and the flags
// that select which launches a step issues.  A graph is reused only while every
// member still has the state it left after the captured step.
unsigned long long state_key(const Ctx& c) {
  unsigned long long k = (unsigned long long)c.allocGen << 16;
  k |= (unsigned long long)c.haveFluid | (unsigned long long)c.haveParcels << 1 | (unsigned long long)c.listsBuilt << 2 |
       (unsigned long long)c.weightsLocal << 3 | (unsigned long long)c.weightsGhost << 4 |
       (unsigned long long)c.planReady << 5 | (unsigned long long)c.spreadValid << 6 | (unsigned long long)c.timing << 7;
  return k;
}

}  // namespace

struct ibmdem_batch {
  int device = 0;
  std::vector<ibmdem_ctx*> cases;
  int lanes = 0;  // 0: one chain per case
  cudaStream_t origin = nullptr;
  std::vector<cudaStream_t> laneStreams;
  std::vector<cudaEvent_t> joins;
  std::vector<cudaEvent_t> inputs;  // per case: its own stream's work before a batch step
  cudaEvent_t fork = nullptr, done = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<long long> launchesPerStep;
  std::vector<unsigned long long> keys;  // member state the captured step leaves
  bool stationary = true;  // the captured step leaves the state it was captured from
  bool dirty = true;
  // the forcing loop of all members in shared launches (ibmdem_batch_set_fused)
  int fused = 0;
  int interpBlock = kBlock;
  void* dDesc = nullptr;
  size_t descBytes = 0;
  ForcingBatch fb;
  cudaEvent_t fork2 = nullptr;
  std::vector<cudaEvent_t> joins2;
  bool capturedFused = false;
  std::string err = "ok";
};

namespace {

int batch_error(ibmdem_batch* b, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  b->err = buf;
  return code;
}

void drop_graph(ibmdem_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
  b->dirty = true;
}

cudaError_t ensure_streams(ibmdem_batch* b, int nLanes) {
  cudaError_t e = cudaSuccess;
  if (!b->origin) e = cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking);
  if (e == cudaSuccess && !b->fork) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  if (e == cudaSuccess && !b->done) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
  if (e == cudaSuccess && !b->fork2) e = cudaEventCreateWithFlags(&b->fork2, cudaEventDisableTiming);
  while (e == cudaSuccess && (int)b->laneStreams.size() < nLanes) {
    cudaStream_t s = nullptr;
    cudaEvent_t j = nullptr, j2 = nullptr;
    e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&j, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&j2, cudaEventDisableTiming);
    if (s) b->laneStreams.push_back(s);
    if (j) b->joins.push_back(j);
    if (j2) b->joins2.push_back(j2);
  }
  while (e == cudaSuccess && b->inputs.size() < b->cases.size()) {
    cudaEvent_t q = nullptr;
    e = cudaEventCreateWithFlags(&q, cudaEventDisableTiming);
    if (q) b->inputs.push_back(q);
  }
  return e;
}

// capture one step of every case into b->graph / b->exec
int capture_batch(ibmdem_batch* b) {
  drop_graph(b);
  const int n = (int)b->cases.size();
  if (n == 0) {
    b->dirty = false;
    return IBMDEM_OK;
  }
  const int nl = b->lanes <= 0 ? n : std::min(b->lanes, n);
  if (cudaSetDevice(b->device) != cudaSuccess) return batch_error(b, IBMDEM_ECUDA, "cudaSetDevice failed");
  cudaError_t e = ensure_streams(b, nl);
  if (e != cudaSuccess) return batch_error(b, IBMDEM_ECUDA, "batch streams: %s", cudaGetErrorString(e));
  // largest case first, onto the chain with the least work so far
  std::vector<int> order(n);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int x, int y) { return case_work(b->cases[x]->c) > case_work(b->cases[y]->c); });
  std::vector<double> load(nl, 0.0);
  std::vector<int> laneOf(n, 0);
  for (int i : order) {
    int best = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    laneOf[i] = best;
    load[best] += case_work(b->cases[i]->c);
  }
  b->launchesPerStep.assign(n, 0);
  // a pending asynchronous field read-out is waited for on the member's own
  // stream (the graph is ordered after it), not inside the capture
  for (ibmdem_ctx* m : b->cases) wait_fields_read(m->c);
  // The forcing loop in shared launches needs every member to run the same
  // number of forcing iterations; the members' descriptor table is uploaded
  // here, before the capture.
  bool useFused = b->fused != 0;
  for (ibmdem_ctx* m : b->cases)
    useFused = useFused && m->c.p.Ns > 0 && m->c.p.Ns == b->cases[0]->c.p.Ns && m->c.runsSized;
  if (useFused) {
    std::vector<Ctx*> members(n);
    for (int i = 0; i < n; ++i) members[i] = &b->cases[i]->c;
    const size_t need = forcing_desc_bytes(members, b->interpBlock);
    if (b->descBytes < need) {
      if (b->dDesc) cudaFree(b->dDesc);
      b->dDesc = nullptr;
      b->descBytes = 0;
      e = cudaMalloc(&b->dDesc, need);
      if (e != cudaSuccess) return batch_error(b, IBMDEM_ENOMEM, "batch table: %s", cudaGetErrorString(e));
      b->descBytes = need;
    }
    e = forcing_desc_upload(members, b->dDesc, b->interpBlock, b->origin, &b->fb);
    if (e != cudaSuccess) return batch_error(b, IBMDEM_ECUDA, "batch table: %s", cudaGetErrorString(e));
  }
  std::vector<unsigned long long> pre(n);
  for (int i = 0; i < n; ++i) pre[i] = state_key(b->cases[i]->c);
  e = cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) return batch_error(b, IBMDEM_ECUDA, "begin capture: %s", cudaGetErrorString(e));
  cudaEventRecord(b->fork, b->origin);
  for (int k = 0; k < nl; ++k) cudaStreamWaitEvent(b->laneStreams[k], b->fork, 0);
  int rc = IBMDEM_OK;
  int failed = -1;
  // one member's part of the step on its chain: the whole step, or the part
  // before (part 1) or after (part 2) the shared forcing loop
  auto member_part = [&](int i, int part) {
    Ctx& c = b->cases[i]->c;
    cudaStream_t own = c.stream;
    bool timing = c.timing;
    c.stream = b->laneStreams[laneOf[i]];
    c.timing = false;
    long long l0 = c.launches;
    int r = part == 0 ? ibmdem_step(b->cases[i], 1)
                      : (part == 1 ? step_before_forcing(b->cases[i]) : step_after_forcing(b->cases[i]));
    b->launchesPerStep[i] += c.launches - l0;
    c.launches = l0;  // counted again per replay
    c.stream = own;
    c.timing = timing;
    return r;
  };
  auto join_lanes = [&](std::vector<cudaEvent_t>& ev) {
    for (int k = 0; k < nl; ++k) {
      cudaEventRecord(ev[k], b->laneStreams[k]);
      cudaStreamWaitEvent(b->origin, ev[k], 0);
    }
  };
  for (int i : order) {
    if ((rc = member_part(i, useFused ? 1 : 0))) {
      failed = i;
      break;
    }
  }
  if (useFused && !rc) {
    // every member's plan and reset done: the forcing iterations of all of
    // them, two launches each, then their images and CloudEvolutionMS
    join_lanes(b->joins);
    const int Ns = b->cases[0]->c.p.Ns;
    for (int it = 0; it < Ns; ++it) launch_forcing_batch(b->fb, it == 0 ? 3 : 0, b->origin);
    b->launchesPerStep[0] += 2ll * Ns;
    cudaEventRecord(b->fork2, b->origin);
    for (int k = 0; k < nl; ++k) cudaStreamWaitEvent(b->laneStreams[k], b->fork2, 0);
    for (int i : order) {
      if ((rc = member_part(i, 2))) {
        failed = i;
        break;
      }
    }
    join_lanes(b->joins2);
  } else {
    join_lanes(b->joins);
  }
  b->capturedFused = useFused;
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(b->origin, &g);
  if (rc || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    if (rc) return batch_error(b, rc, "case %d: %s", failed, b->cases[failed]->c.err.c_str());
    return batch_error(b, IBMDEM_ECUDA, "end capture: %s", cudaGetErrorString(e));
  }
  e = cudaGraphInstantiate(&b->exec, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    b->exec = nullptr;
    return batch_error(b, IBMDEM_ECUDA, "graph instantiate: %s", cudaGetErrorString(e));
  }
  b->graph = g;
  b->keys.resize(n);
  for (int i = 0; i < n; ++i) b->keys[i] = state_key(b->cases[i]->c);
  b->stationary = b->keys == pre;
  b->dirty = false;
  return IBMDEM_OK;
}

int launch_batch(ibmdem_batch* b, int nsteps) {
  for (size_t i = 0; !b->dirty && i < b->cases.size(); ++i)
    if (state_key(b->cases[i]->c) != b->keys[i]) b->dirty = true;
  if (b->dirty) {
    int rc = capture_batch(b);
    if (rc) return rc;
  }
  if (b->cases.empty() || nsteps <= 0) return IBMDEM_OK;
  // order the batch after what each case's own stream already holds
  for (size_t i = 0; i < b->cases.size(); ++i) {
    wait_fields_read(b->cases[i]->c);
    cudaEventRecord(b->inputs[i], b->cases[i]->c.stream);
    cudaStreamWaitEvent(b->origin, b->inputs[i], 0);
  }
  for (int s = 0; s < nsteps; ++s) {
    // a step that changes the host state it was captured from (the first one
    // after a member's state changed) is replayed once, then captured again
    // from the state it left; the replays are ordered on the origin stream
    if (b->dirty) {
      int rc = capture_batch(b);
      if (rc) return rc;
    }
    cudaError_t e = cudaGraphLaunch(b->exec, b->origin);
    if (e != cudaSuccess) return batch_error(b, IBMDEM_ECUDA, "graph launch: %s", cudaGetErrorString(e));
    for (size_t i = 0; i < b->cases.size(); ++i) b->cases[i]->c.launches += b->launchesPerStep[i];
    if (!b->stationary) b->dirty = true;
  }
  // and each case's own stream after the batch
  cudaEventRecord(b->done, b->origin);
  for (size_t i = 0; i < b->cases.size(); ++i) cudaStreamWaitEvent(b->cases[i]->c.stream, b->done, 0);
  return IBMDEM_OK;
}

}  // namespace

// ---- request server ----------------------------------------------------------

namespace {

struct Request {
  long long id = 0;
  ibmdem_params p{};
  int np = 0, nMS = 0, nsteps = 0;
  const ibmdem_parcel* parts = nullptr;     // borrowed until admission
  const ibmdem_multisphere* bodies = nullptr;
  const double *u = nullptr, *v = nullptr, *w = nullptr;
  bool keepParcels = false;
  long long bytes = 0;
  bool reserved = false;  // bytes and parcels counted in the server's in-use totals
  double tSubmit = 0, tAdmit = 0, tDone = 0;
  int state = 0;  // 0 queued, 1 running, 2 done, < 0 failed (status code)
  ibmdem_ctx* ctx = nullptr;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t done = nullptr;
  std::vector<ibmdem_parcel> outParts;
  int outNp = 0, outNl = 0;
  std::vector<ibmdem_multisphere> outBodies;
  std::string err;
};

}  // namespace

struct ibmdem_server {
  int device = 0;
  long long budget = 0;
  int maxActive = 0;
  long long inUse = 0;
  long long workLimit = 0;  // parcels in flight (0: no limit)
  long long workInUse = 0;
  int policy = 0;          // 0: arrival order, 1: least work first
  double ageLimit = 0.0;   // policy 1: a request queued this long (s) goes first (0: never)
  long long nextId = 1;
  std::deque<Request*> queue;
  std::vector<Request*> running;
  std::unordered_map<long long, Request*> all;
  std::string err = "ok";
};

namespace {

void release_device(ibmdem_server* s, Request* r) {
  if (r->exec) cudaGraphExecDestroy(r->exec);
  if (r->graph) cudaGraphDestroy(r->graph);
  r->exec = nullptr;
  r->graph = nullptr;
  if (r->ctx) ibmdem_destroy(r->ctx);
  r->ctx = nullptr;
  if (r->done) cudaEventDestroy(r->done);
  r->done = nullptr;
  if (r->stream) cudaStreamDestroy(r->stream);
  r->stream = nullptr;
  if (r->reserved) {
    s->inUse -= r->bytes;
    s->workInUse -= r->np;
  }
  r->reserved = false;
}

int fail(ibmdem_server* s, Request* r, int code) {
  if (r->ctx && r->err.empty()) r->err = r->ctx->c.err;
  release_device(s, r);
  r->state = code < 0 ? code : IBMDEM_ECUDA;
  r->tDone = now_s();
  return r->state;
}

// create the case on its own stream, initialise it, capture its step and queue
// all of its steps
int admit(ibmdem_server* s, Request* r) {
  r->tAdmit = now_s();
  s->inUse += r->bytes;
  s->workInUse += r->np;
  r->reserved = true;
  r->state = 1;
  auto cu = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess) fmt_err(r->err, "%s: %s", what, cudaGetErrorString(e));
    return e == cudaSuccess;
  };
  if (!cu(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking), "stream")) return fail(s, r, IBMDEM_ECUDA);
  if (!cu(cudaEventCreateWithFlags(&r->done, cudaEventDisableTiming), "event")) return fail(s, r, IBMDEM_ECUDA);
  int rc = create_on_stream(&r->p, s->device, r->stream, &r->ctx);
  if (rc) {
    fmt_err(r->err, "case creation failed (%d)", rc);
    return fail(s, r, rc);
  }
  Ctx& c = r->ctx->c;
  if (r->u) {
    rc = ibmdem_set_fluid(r->ctx, r->u, r->v, r->w);
  } else {
    // the fields were zeroed at creation: a fluid at rest
    c.haveFluid = true;
  }
  if (!rc) rc = ibmdem_set_bodies(r->ctx, r->nMS, r->bodies);
  if (!rc) rc = ibmdem_set_parcels(r->ctx, r->np, r->parts);
  if (!rc) rc = ibmdem_InitializationDEM(r->ctx);
  if (rc) return fail(s, r, rc);
  // account what the case actually holds (the run arrays follow the counted
  // touched nodes, the admission estimate assumed a typical density)
  s->inUse += (long long)c.bytes - r->bytes;
  r->bytes = (long long)c.bytes;
  r->parts = nullptr;
  r->bodies = nullptr;
  r->u = r->v = r->w = nullptr;
  // capture one step and queue the rest as replays; a step that leaves another
  // host state than it was captured from is replayed once and captured again
  int left = r->nsteps;
  for (int attempt = 0; left > 0; ++attempt) {
    const unsigned long long pre = state_key(c);
    if (!cu(cudaStreamBeginCapture(r->stream, cudaStreamCaptureModeRelaxed), "begin capture"))
      return fail(s, r, IBMDEM_ECUDA);
    long long l0 = c.launches;
    rc = ibmdem_step(r->ctx, 1);
    long long perStep = c.launches - l0;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(r->stream, &g);
    if (rc || e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      if (!rc) cu(e, "end capture");
      return fail(s, r, rc ? rc : IBMDEM_ECUDA);
    }
    if (r->exec) cudaGraphExecDestroy(r->exec);  // freed once its queued replays finish
    if (r->graph) cudaGraphDestroy(r->graph);
    r->exec = nullptr;
    r->graph = g;
    if (!cu(cudaGraphInstantiate(&r->exec, g, 0), "graph instantiate")) return fail(s, r, IBMDEM_ECUDA);
    c.launches = l0;
    const bool stationary = state_key(c) == pre;
    if (!stationary && attempt > 0) {
      fmt_err(r->err, "the step does not return to the host state it was captured from");
      return fail(s, r, IBMDEM_EINVAL);
    }
    const int k = stationary ? left : 1;
    for (int q = 0; q < k; ++q)
      if (!cu(cudaGraphLaunch(r->exec, r->stream), "graph launch")) return fail(s, r, IBMDEM_ECUDA);
    c.launches += perStep * k;
    left -= k;
  }
  if (!cu(cudaEventRecord(r->done, r->stream), "event record")) return fail(s, r, IBMDEM_ECUDA);
  s->running.push_back(r);
  return IBMDEM_OK;
}

// read back a finished case and return its memory
void retire(ibmdem_server* s, Request* r) {
  r->tDone = now_s();
  int rc = ibmdem_synchronize(r->ctx);
  if (!rc) {
    int nMS = 0;
    rc = ibmdem_get_bodies(r->ctx, nullptr, 0, &nMS);
    r->outBodies.resize(nMS);
    if (!rc && nMS) rc = ibmdem_get_bodies(r->ctx, r->outBodies.data(), nMS, &nMS);
  }
  if (!rc && r->keepParcels) {
    rc = ibmdem_get_parcels(r->ctx, nullptr, 0, &r->outNp, &r->outNl);
    r->outParts.resize(r->outNp);
    if (!rc && r->outNp) rc = ibmdem_get_parcels(r->ctx, r->outParts.data(), r->outNp, &r->outNp, &r->outNl);
  }
  if (rc) r->err = r->ctx->c.err;
  release_device(s, r);
  r->state = rc ? rc : 2;
}

}  // namespace

extern "C" {

int ibmdem_batch_create(int32_t device, ibmdem_batch** out) {
  if (!out) return IBMDEM_EINVAL;
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return IBMDEM_ECUDA;
  ibmdem_batch* b = new (std::nothrow) ibmdem_batch();
  if (!b) return IBMDEM_ENOMEM;
  b->device = device;
  *out = b;
  return IBMDEM_OK;
}

int ibmdem_batch_destroy(ibmdem_batch* b) {
  if (!b) return IBMDEM_EINVAL;
  cudaSetDevice(b->device);
  if (b->origin) cudaStreamSynchronize(b->origin);
  drop_graph(b);
  for (cudaStream_t s : b->laneStreams) cudaStreamDestroy(s);
  for (cudaEvent_t e : b->joins) cudaEventDestroy(e);
  for (cudaEvent_t e : b->joins2) cudaEventDestroy(e);
  for (cudaEvent_t e : b->inputs) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->fork2) cudaEventDestroy(b->fork2);
  if (b->dDesc) cudaFree(b->dDesc);
  if (b->done) cudaEventDestroy(b->done);
  if (b->origin) cudaStreamDestroy(b->origin);
  delete b;
  return IBMDEM_OK;
}

const char* ibmdem_batch_last_error(const ibmdem_batch* b) { return b ? b->err.c_str() : "null batch"; }

int ibmdem_batch_add(ibmdem_batch* b, ibmdem_ctx* ctx) {
  if (!b || !ctx) return IBMDEM_EINVAL;
  if (ctx->c.device != b->device) return batch_error(b, IBMDEM_EINVAL, "case is on device %d, batch on %d",
                                                     ctx->c.device, b->device);
  if (std::find(b->cases.begin(), b->cases.end(), ctx) != b->cases.end())
    return batch_error(b, IBMDEM_EINVAL, "case already in the batch");
  b->cases.push_back(ctx);
  drop_graph(b);
  return IBMDEM_OK;
}

int ibmdem_batch_set_lanes(ibmdem_batch* b, int32_t lanes) {
  if (!b || lanes < 0) return IBMDEM_EINVAL;
  if (lanes != b->lanes) {
    b->lanes = lanes;
    drop_graph(b);
  }
  return IBMDEM_OK;
}

int ibmdem_batch_set_fused(ibmdem_batch* b, int32_t fused, int32_t interp_block) {
  if (!b || (fused != 0 && fused != 1) || (interp_block != 128 && interp_block != 256)) return IBMDEM_EINVAL;
  if (fused != b->fused || interp_block != b->interpBlock) {
    b->fused = fused;
    b->interpBlock = interp_block;
    drop_graph(b);
  }
  return IBMDEM_OK;
}

int ibmdem_batch_get_config(const ibmdem_batch* b, int32_t* lanes, int32_t* fused, int32_t* interp_block) {
  if (!b) return IBMDEM_EINVAL;
  if (lanes) *lanes = b->lanes;
  if (fused) *fused = b->fused;
  if (interp_block) *interp_block = b->interpBlock;
  return IBMDEM_OK;
}

int ibmdem_batch_step(ibmdem_batch* b, int32_t nsteps) {
  if (!b || nsteps < 0) return IBMDEM_EINVAL;
  if (cudaSetDevice(b->device) != cudaSuccess) return batch_error(b, IBMDEM_ECUDA, "cudaSetDevice failed");
  return launch_batch(b, nsteps);
}

int ibmdem_batch_synchronize(ibmdem_batch* b, int32_t* failed_case) {
  if (!b) return IBMDEM_EINVAL;
  if (failed_case) *failed_case = -1;
  cudaSetDevice(b->device);
  if (b->origin) {
    cudaError_t e = cudaStreamSynchronize(b->origin);
    if (e != cudaSuccess) return batch_error(b, IBMDEM_ECUDA, "batch stream: %s", cudaGetErrorString(e));
  }
  for (size_t i = 0; i < b->cases.size(); ++i) {
    int rc = ibmdem_synchronize(b->cases[i]);
    if (rc) {
      if (failed_case) *failed_case = (int32_t)i;
      return batch_error(b, rc, "case %zu: %s", i, b->cases[i]->c.err.c_str());
    }
  }
  return IBMDEM_OK;
}

int ibmdem_batch_autotune(ibmdem_batch* b, int32_t trial_steps, int32_t* lanes_out) {
  if (!b || trial_steps < 1) return IBMDEM_EINVAL;
  const int n = (int)b->cases.size();
  if (n == 0) {
    if (lanes_out) *lanes_out = 0;
    return IBMDEM_OK;
  }
  cudaSetDevice(b->device);
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  // one trial: capture the configuration, a warm-up step, then trial_steps timed
  auto trial = [&](int lanes, int fused, int block, float* ms) {
    b->lanes = lanes;
    b->fused = fused;
    b->interpBlock = block;
    drop_graph(b);
    int rc = launch_batch(b, 1);
    if (rc) return rc;
    cudaEventRecord(t0, b->origin);
    rc = launch_batch(b, trial_steps);
    if (rc) return rc;
    cudaEventRecord(t1, b->origin);
    if (cudaEventSynchronize(t1) != cudaSuccess) return batch_error(b, IBMDEM_ECUDA, "autotune trial failed");
    cudaEventElapsedTime(ms, t0, t1);
    return IBMDEM_OK;
  };
  // first the chain count with each member's own forcing launches, then the
  // shared forcing launches (both interpolation block sizes) around the best
  // chain counts
  std::vector<int> cands;
  for (int k : {n, 128, 64, 32, 16, 8, 4, 2, 1})
    if (k <= n && std::find(cands.begin(), cands.end(), k) == cands.end()) cands.push_back(k);
  int best = n, bestFused = 0, bestBlock = kBlock;
  float bestMs = 0.f;
  bool any = false;
  int rc = IBMDEM_OK;
  std::vector<std::pair<float, int>> own;
  for (int k : cands) {
    float ms = 0.f;
    if ((rc = trial(k, 0, kBlock, &ms))) break;
    own.push_back({ms, k});
    if (!any || ms < bestMs) {
      bestMs = ms;
      best = k;
      any = true;
    }
  }
  if (!rc) {
    std::sort(own.begin(), own.end());
    for (size_t q = 0; q < own.size() && q < 2 && !rc; ++q)
      for (int block : {kBlock, 128}) {
        float ms = 0.f;
        if ((rc = trial(own[q].second, 1, block, &ms))) break;
        if (ms < bestMs) {
          bestMs = ms;
          best = own[q].second;
          bestFused = 1;
          bestBlock = block;
        }
      }
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (rc) return rc;
  b->lanes = best;
  b->fused = bestFused;
  b->interpBlock = bestBlock;
  drop_graph(b);
  if (lanes_out) *lanes_out = best;
  return IBMDEM_OK;
}

int ibmdem_server_create(int32_t device, int64_t hbm_budget, int32_t max_active, ibmdem_server** out) {
  if (!out || hbm_budget <= 0 || max_active < 1) return IBMDEM_EINVAL;
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return IBMDEM_ECUDA;
  ibmdem_server* s = new (std::nothrow) ibmdem_server();
  if (!s) return IBMDEM_ENOMEM;
  s->device = device;
  s->budget = hbm_budget;
  s->maxActive = max_active;
  *out = s;
  return IBMDEM_OK;
}

int ibmdem_server_destroy(ibmdem_server* s) {
  if (!s) return IBMDEM_EINVAL;
  cudaSetDevice(s->device);
  for (Request* r : s->running) {
    if (r->stream) cudaStreamSynchronize(r->stream);
    release_device(s, r);
  }
  for (auto& kv : s->all) delete kv.second;
  delete s;
  return IBMDEM_OK;
}

const char* ibmdem_server_last_error(const ibmdem_server* s) { return s ? s->err.c_str() : "null server"; }

int ibmdem_server_submit(ibmdem_server* s, const ibmdem_params* p, int32_t np, const ibmdem_parcel* parts,
                         int32_t nMS, const ibmdem_multisphere* bodies, const double* u, const double* v,
                         const double* w, int32_t nsteps, int32_t keep_parcels, int64_t* id) {
  if (!s || !p || !id || np < 0 || nMS < 0 || nsteps < 0 || (np > 0 && !parts) || (nMS > 0 && !bodies) ||
      ((u == nullptr) != (v == nullptr)) || ((u == nullptr) != (w == nullptr)))
    return IBMDEM_EINVAL;
  int64_t bytes = 0;
  int rc = ibmdem_case_bytes(p, np, parts, nMS, &bytes);
  if (rc) {
    fmt_err(s->err, "unsupported case parameters (%d)", rc);
    return rc;
  }
  if (bytes > s->budget) {
    fmt_err(s->err, "case needs %lld bytes, above the whole budget of %lld", (long long)bytes, s->budget);
    return IBMDEM_ERANGE;
  }
  Request* r = new (std::nothrow) Request();
  if (!r) return IBMDEM_ENOMEM;
  r->id = s->nextId++;
  r->p = *p;
  r->np = np;
  r->parts = parts;
  r->nMS = nMS;
  r->bodies = bodies;
  r->u = u;
  r->v = v;
  r->w = w;
  r->nsteps = nsteps;
  r->keepParcels = keep_parcels != 0;
  r->bytes = bytes;
  r->tSubmit = now_s();
  s->queue.push_back(r);
  s->all[r->id] = r;
  *id = r->id;
  return IBMDEM_OK;
}

int ibmdem_server_poll(ibmdem_server* s, int32_t* pending) {
  if (!s) return IBMDEM_EINVAL;
  cudaSetDevice(s->device);
  // retire the cases whose last step has completed
  for (size_t i = 0; i < s->running.size();) {
    Request* r = s->running[i];
    cudaError_t q = cudaEventQuery(r->done);
    if (q == cudaErrorNotReady) {
      ++i;
      continue;
    }
    if (q == cudaSuccess) {
      retire(s, r);
    } else {
      fmt_err(r->err, "case failed on the device: %s", cudaGetErrorString(q));
      fail(s, r, IBMDEM_ECUDA);
    }
    s->running[i] = s->running.back();
    s->running.pop_back();
  }
  // admit while the budget, the slots and the work limit allow (the work
  // limit always lets one case run): the oldest request, or under the
  // least-work policy the one with the fewest marker-steps unless one has
  // waited past the age limit (then the oldest of those)
  while (!s->queue.empty() && (int)s->running.size() < s->maxActive) {
    size_t pick = 0;
    if (s->policy == 1) {
      const double t = now_s();
      const bool aged = s->ageLimit > 0.0 && t - s->queue.front()->tSubmit > s->ageLimit;
      if (!aged)
        for (size_t q = 1; q < s->queue.size(); ++q)
          if ((long long)s->queue[q]->np * s->queue[q]->nsteps < (long long)s->queue[pick]->np * s->queue[pick]->nsteps)
            pick = q;
    }
    Request* r = s->queue[pick];
    if (s->inUse + r->bytes > s->budget ||
        (s->workLimit > 0 && !s->running.empty() && s->workInUse + r->np > s->workLimit))
      break;
    s->queue.erase(s->queue.begin() + (long)pick);
    admit(s, r);
  }
  if (pending) *pending = (int32_t)(s->queue.size() + s->running.size());
  return IBMDEM_OK;
}

int ibmdem_server_status(ibmdem_server* s, int64_t id, int32_t* state, double* latency_s, double* queue_s) {
  if (!s) return IBMDEM_EINVAL;
  auto it = s->all.find(id);
  if (it == s->all.end()) return IBMDEM_EINVAL;
  Request* r = it->second;
  if (state) *state = r->state;
  if (latency_s) *latency_s = r->tDone > 0 ? r->tDone - r->tSubmit : 0.0;
  if (queue_s) *queue_s = r->tAdmit > 0 ? r->tAdmit - r->tSubmit : 0.0;
  if (r->state < 0) s->err = r->err;
  return IBMDEM_OK;
}

int ibmdem_server_result(ibmdem_server* s, int64_t id, ibmdem_parcel* parts, int32_t cap_parts, int32_t* np,
                         int32_t* nlocal, ibmdem_multisphere* bodies, int32_t cap_bodies, int32_t* nMS) {
  if (!s) return IBMDEM_EINVAL;
  auto it = s->all.find(id);
  if (it == s->all.end()) return IBMDEM_EINVAL;
  Request* r = it->second;
  if (r->state < 0) {
    s->err = r->err;
    return r->state;
  }
  if (r->state != 2) {
    fmt_err(s->err, "request %lld has not finished", (long long)id);
    return IBMDEM_ESTATE;
  }
  if (np) *np = r->outNp;
  if (nlocal) *nlocal = r->outNl;
  if (nMS) *nMS = (int32_t)r->outBodies.size();
  if (parts && !r->outParts.empty())
    std::memcpy(parts, r->outParts.data(), sizeof(ibmdem_parcel) * std::min<size_t>(r->outParts.size(), cap_parts));
  if (bodies && !r->outBodies.empty())
    std::memcpy(bodies, r->outBodies.data(),
                sizeof(ibmdem_multisphere) * std::min<size_t>(r->outBodies.size(), cap_bodies));
  return IBMDEM_OK;
}

int ibmdem_server_release(ibmdem_server* s, int64_t id) {
  if (!s) return IBMDEM_EINVAL;
  auto it = s->all.find(id);
  if (it == s->all.end()) return IBMDEM_EINVAL;
  Request* r = it->second;
  if (r->state == 0 || r->state == 1) {
    fmt_err(s->err, "request %lld is still queued or running", (long long)id);
    return IBMDEM_ESTATE;
  }
  s->all.erase(it);
  delete r;
  return IBMDEM_OK;
}

int ibmdem_server_set_policy(ibmdem_server* s, int32_t policy, double age_limit_s) {
  if (!s || (policy != 0 && policy != 1) || !(age_limit_s >= 0.0)) return IBMDEM_EINVAL;
  s->policy = policy;
  s->ageLimit = age_limit_s;
  return IBMDEM_OK;
}

int ibmdem_server_set_work_limit(ibmdem_server* s, int64_t parcels) {
  if (!s || parcels < 0) return IBMDEM_EINVAL;
  s->workLimit = parcels;
  return IBMDEM_OK;
}

int ibmdem_server_memory(const ibmdem_server* s, int64_t* in_use, int64_t* budget) {
  if (!s) return IBMDEM_EINVAL;
  if (in_use) *in_use = s->inUse;
  if (budget) *budget = s->budget;
  return IBMDEM_OK;
}

}  // extern "C"
