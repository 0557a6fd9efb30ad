// Continuous-batching server (split_server_*): host C++ over the batch entry
// points.  The reference has no serving layer; its only caller segments one
// image per run (samples/src/main.cu:154-372).
//
// Requests (an RGB8 image in host memory, its K, iteration count and initial
// centroids, and host buffers for the results) are submitted from any thread.
// One worker thread per server:
//   * admits waiting requests in arrival order while their device footprint
//     fits the HBM budget (a request never overtakes an earlier one);
//   * packs every admitted request into the next batch (up to a pixel cap,
//     at least one request) while fewer than `max_inflight` batches are on
//     the device;
//   * stages a batch on three streams: uploads into the batch's resident
//     arena, the batch's launch sequence (split_batch_run), downloads of the
//     results into the callers' host buffers, joined by events;
//   * completes a batch's requests when its downloads have landed, returns
//     their footprint to the budget and queues their completions for
//     split_server_poll.
// Each in-flight slot owns a resident arena (RGB, centroids, labels, normals
// and the workspace with union-find and merge state) that its batches bind
// to, so serving allocates device memory only when an arena has to grow
// (split_server_reserve grows them up front).  All batches compute on one
// stream: the k-means stage is a cooperative grid that fills the GPU, and a
// second one beside it would contend for residency; the copy streams overlap
// both directions of host traffic with the compute.
//
// Each request's results are independent of what shares its batch (per-image
// tiles, reduction trees and label spaces), so a request gives the same
// results alone and in any mix.
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"

namespace sg {
namespace srv {

using Clock = std::chrono::steady_clock;

constexpr size_t kDefaultBudget = size_t(40) << 30;
constexpr int64_t kDefaultMaxBatchPixels = int64_t(64) << 20;
constexpr int64_t kGranule = 64;   // batch arenas start every image on 64 pixels

inline int64_t rounded(int64_t px) { return (px + kGranule - 1) / kGranule * kGranule; }

struct Req {
  split_request r;
  uint64_t ticket;
  Clock::time_point submitted;
  int64_t pixels;
  size_t footprint;
};

// FIFO admission under a byte budget and batch formation under a pixel cap.
// Plain host logic (no CUDA), shared by the worker and the host-side test
// entry point split_server_admission_test.
struct Admission {
  size_t budget = 0, in_use = 0, peak = 0;
  std::deque<Req> waiting;
  std::vector<Req> admitted;

  // waiting -> admitted while the head fits; returns how many were admitted
  int admit() {
    int n = 0;
    while (!waiting.empty() && in_use + waiting.front().footprint <= budget) {
      in_use += waiting.front().footprint;
      admitted.push_back(waiting.front());
      waiting.pop_front();
      ++n;
    }
    if (in_use > peak) peak = in_use;
    return n;
  }
  // the admitted requests, in order, that fit the pixel cap (the first one
  // always, so an image larger than the cap still progresses); the rest stay
  std::vector<Req> take(int64_t max_pixels) {
    std::vector<Req> out, keep;
    int64_t px = 0;
    for (Req& q : admitted) {
      if (out.empty() || px + q.pixels <= max_pixels) {
        px += q.pixels;
        out.push_back(q);
      } else {
        keep.push_back(q);
      }
    }
    admitted.swap(keep);
    return out;
  }
  void release(const std::vector<Req>& rs) {
    for (const Req& q : rs) in_use -= q.footprint;
  }
};

// Resident device buffers of one in-flight slot (grow-only).
struct Slot {
  uint8_t* rgb = nullptr;
  float* cent = nullptr;
  int32_t* cl = nullptr;
  int32_t* seg = nullptr;
  float* nrm = nullptr;
  void* ws = nullptr;
  int64_t px = 0, cf = 0;
  size_t wsb = 0;

  void free_all() {
    cudaFree(rgb);
    cudaFree(cent);
    cudaFree(cl);
    cudaFree(seg);
    cudaFree(nrm);
    cudaFree(ws);
    rgb = nullptr;
    cent = nullptr;
    cl = seg = nullptr;
    nrm = nullptr;
    ws = nullptr;
    px = cf = 0;
    wsb = 0;
  }
  // Grows the buffers to the given sizes.  A new workspace is zero-filled on
  // `st`, the stream the batch is then bound on, so the fill is ordered
  // before the bind's uploads (the server's streams do not synchronise with
  // the legacy default stream, where a plain cudaMemset would run).
  int ensure(int64_t need_px, int64_t need_cf, size_t need_wsb, bool normals, cudaStream_t st) {
    if (need_px > px) {
      cudaFree(rgb);
      cudaFree(cl);
      cudaFree(seg);
      cudaFree(nrm);
      rgb = nullptr;
      cl = seg = nullptr;
      nrm = nullptr;
      px = 0;
      SG_CUDA_TRY(cudaMalloc(&rgb, (size_t)need_px * 3));
      SG_CUDA_TRY(cudaMalloc(&cl, (size_t)need_px * 4));
      SG_CUDA_TRY(cudaMalloc(&seg, (size_t)need_px * 4));
      if (normals) SG_CUDA_TRY(cudaMalloc(&nrm, (size_t)need_px * 12));
      px = need_px;
    }
    if (need_cf > cf) {
      cudaFree(cent);
      cent = nullptr;
      cf = 0;
      SG_CUDA_TRY(cudaMalloc(&cent, (size_t)need_cf * 4));
      cf = need_cf;
    }
    if (need_wsb > wsb) {
      cudaFree(ws);
      ws = nullptr;
      wsb = 0;
      SG_CUDA_TRY(cudaMalloc(&ws, need_wsb));
      // a workspace is zero-filled once, when it is made
      SG_CUDA_TRY(cudaMemsetAsync(ws, 0, need_wsb, st));
      wsb = need_wsb;
    }
    return SPLIT_OK;
  }
};

struct Flight {
  std::vector<Req> reqs;
  split_batch* plan = nullptr;
  cudaEvent_t done = nullptr;
  int slot = 0;
  int status = SPLIT_OK;   // a launch error completes every request with it
};

// Device bytes one pixel of a batch holds: the arenas (RGB8, two label
// planes, normals) plus the batch workspace of a 1024 x 1024 probe image
// clustered more than once (so that it keeps span sums), per pixel, rounded
// up.
size_t bytes_per_pixel(const split_pipeline_params& p) {
  split_batch_image im{1024, 1024, 64, 2};
  split_batch* b = nullptr;
  if (split_batch_create(&im, 1, &p, &b) != SPLIT_OK) return 0;
  const size_t ws = split_batch_workspace_size(b);
  const int64_t px = split_batch_arena_pixels(b);
  split_batch_destroy(b);
  const size_t arenas = 3 + 4 + 4 + (p.compute_normals ? 12 : 0);
  return arenas + (ws + (size_t)px - 1) / (size_t)px;
}

}  // namespace srv
}  // namespace sg

using namespace sg;
using namespace sg::srv;

struct split_server {
  split_server_config cfg{};
  size_t bpp = 0;
  cudaStream_t h2d = nullptr, compute = nullptr, d2h = nullptr;
  std::vector<Slot> slots;
  int next_slot = 0;
  std::mutex mu;
  std::condition_variable work_cv, done_cv;
  Admission adm;                 // guarded by mu
  std::deque<split_completion> done;   // guarded by mu
  std::deque<Flight> flights;    // worker thread only
  int nflights = 0;              // guarded by mu (flights.size() for other threads)
  uint64_t next_ticket = 1, submitted = 0, completed = 0, batches = 0;
  bool stop = false;
  std::thread worker;
};

namespace {

void complete(split_server* s, Flight& f, int status) {
  const Clock::time_point now = Clock::now();
  std::vector<split_completion> out;
  out.reserve(f.reqs.size());
  for (const Req& q : f.reqs) {
    split_completion c{};
    c.ticket = q.ticket;
    c.user = q.r.user;
    c.status = status;
    c.pixels = q.pixels;
    c.latency_ms = std::chrono::duration<double, std::milli>(now - q.submitted).count();
    out.push_back(c);
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->adm.release(f.reqs);
    for (const split_completion& c : out) s->done.push_back(c);
    s->completed += out.size();
    s->nflights -= 1;
  }
  s->done_cv.notify_all();
  s->work_cv.notify_all();
}

// Queue one batch: plan, arena, bind, uploads, run, downloads.
int stage(split_server* s, Flight& f) {
  const split_server_config& c = s->cfg;
  const int n = (int)f.reqs.size();
  std::vector<split_batch_image> ims(n);
  for (int i = 0; i < n; ++i)
    ims[i] = {f.reqs[i].r.width, f.reqs[i].r.height, f.reqs[i].r.nclusters,
              f.reqs[i].r.kmeans_iters};
  SG_TRY(split_batch_create(ims.data(), n, &c.params, &f.plan));
  Slot& sl = s->slots[f.slot];
  SG_TRY(sl.ensure(split_batch_arena_pixels(f.plan), split_batch_centroid_floats(f.plan),
                   split_batch_workspace_size(f.plan), c.params.compute_normals != 0, s->h2d));
  SG_TRY(split_batch_bind(f.plan, sl.rgb, sl.cent, sl.cl, sl.seg, sl.nrm, sl.ws, sl.wsb, s->h2d));
  const int dim = c.params.dim;
  for (int i = 0; i < n; ++i) {
    const split_request& r = f.reqs[i].r;
    const int64_t off = split_batch_pixel_offset(f.plan, i);
    const int64_t coff = split_batch_centroid_offset(f.plan, i);
    SG_CUDA_TRY(cudaMemcpyAsync(sl.rgb + 3 * off, r.rgb, (size_t)3 * f.reqs[i].pixels,
                                cudaMemcpyHostToDevice, s->h2d));
    SG_CUDA_TRY(cudaMemcpyAsync(sl.cent + coff, r.centroids, sizeof(float) * dim * r.nclusters,
                                cudaMemcpyHostToDevice, s->h2d));
  }
  cudaEvent_t up = nullptr, ran = nullptr;
  SG_CUDA_TRY(cudaEventCreateWithFlags(&up, cudaEventDisableTiming));
  SG_CUDA_TRY(cudaEventCreateWithFlags(&ran, cudaEventDisableTiming));
  int st = SPLIT_OK;
  auto run = [&]() -> int {
    SG_CUDA_TRY(cudaEventRecord(up, s->h2d));
    SG_CUDA_TRY(cudaStreamWaitEvent(s->compute, up, 0));
    SG_TRY(split_batch_run(f.plan, s->compute));
    SG_CUDA_TRY(cudaEventRecord(ran, s->compute));
    SG_CUDA_TRY(cudaStreamWaitEvent(s->d2h, ran, 0));
    for (int i = 0; i < n; ++i) {
      const split_request& r = f.reqs[i].r;
      const int64_t px = f.reqs[i].pixels;
      const int64_t off = split_batch_pixel_offset(f.plan, i);
      const int64_t coff = split_batch_centroid_offset(f.plan, i);
      SG_CUDA_TRY(cudaMemcpyAsync(r.segment_labels, sl.seg + off, sizeof(int32_t) * px,
                                  cudaMemcpyDeviceToHost, s->d2h));
      if (r.cluster_labels)
        SG_CUDA_TRY(cudaMemcpyAsync(r.cluster_labels, sl.cl + off, sizeof(int32_t) * px,
                                    cudaMemcpyDeviceToHost, s->d2h));
      if (r.centroids_out)
        SG_CUDA_TRY(cudaMemcpyAsync(r.centroids_out, sl.cent + coff,
                                    sizeof(float) * dim * r.nclusters, cudaMemcpyDeviceToHost,
                                    s->d2h));
      if (r.normals && sl.nrm)
        SG_CUDA_TRY(cudaMemcpyAsync(r.normals, sl.nrm + 3 * off, sizeof(float) * 3 * px,
                                    cudaMemcpyDeviceToHost, s->d2h));
    }
    SG_CUDA_TRY(cudaEventCreateWithFlags(&f.done, cudaEventDisableTiming));
    SG_CUDA_TRY(cudaEventRecord(f.done, s->d2h));
    return SPLIT_OK;
  };
  st = run();
  // the events are only waited on through streams that were enqueued
  // above: destroying them now is safe (CUDA defers the release)
  cudaEventDestroy(up);
  cudaEventDestroy(ran);
  return st;
}

// Finish the oldest flight once its downloads have landed.
void finish(split_server* s, Flight& f) {
  int st = f.status;
  if (st == SPLIT_OK) {
    int dev_status = SPLIT_OK;
    // the batch's stage errors, folded into its workspace status word
    // (the read clears the word on d2h: wait for that before the slot is
    // bound again, so it cannot erase an error of the slot's next batch)
    if (split_workspace_status(s->slots[f.slot].ws, s->d2h, &dev_status) != SPLIT_OK ||
        cudaStreamSynchronize(s->d2h) != cudaSuccess)
      st = SPLIT_ERR_CUDA;
    else
      st = dev_status;
  }
  if (f.done) cudaEventDestroy(f.done);
  if (f.plan) split_batch_destroy(f.plan);
  f.done = nullptr;
  f.plan = nullptr;
  complete(s, f, st);
}

void worker_main(split_server* s) {
  cudaSetDevice(s->cfg.device);
  for (;;) {
    std::vector<Req> take;
    bool idle = false;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->adm.admit();
      const bool room = (int)s->flights.size() < s->cfg.max_inflight;
      if (!s->adm.admitted.empty() && room) {
        take = s->adm.take(s->cfg.max_batch_pixels);
        s->nflights += 1;
        s->batches += 1;
      } else if (s->flights.empty()) {
        if (s->stop && s->adm.waiting.empty() && s->adm.admitted.empty()) break;
        idle = true;
      }
      if (idle) {
        s->work_cv.wait(lk);
        continue;
      }
    }
    if (!take.empty()) {
      Flight f;
      f.reqs = std::move(take);
      f.slot = s->next_slot;
      s->next_slot = (s->next_slot + 1) % s->cfg.max_inflight;
      f.status = stage(s, f);
      s->flights.push_back(std::move(f));
      continue;
    }
    // collect: the oldest flight first (slots are reused in launch order)
    Flight& f = s->flights.front();
    if (f.status != SPLIT_OK || !f.done) {
      Flight g = std::move(f);
      s->flights.pop_front();
      finish(s, g);
      continue;
    }
    cudaError_t q = cudaEventQuery(f.done);
    if (q == cudaErrorNotReady) {
      const bool full = (int)s->flights.size() >= s->cfg.max_inflight;
      if (full) {
        q = cudaEventSynchronize(f.done);
      } else {
        // room for another batch: wake for a new submission or poll again
        std::unique_lock<std::mutex> lk(s->mu);
        s->work_cv.wait_for(lk, std::chrono::microseconds(100));
        continue;
      }
    }
    if (q != cudaSuccess && q != cudaErrorNotReady) f.status = SPLIT_ERR_CUDA;
    Flight g = std::move(f);
    s->flights.pop_front();
    finish(s, g);
  }
}

}  // namespace

extern "C" size_t split_server_bytes_per_pixel(const split_pipeline_params* params) {
  return params ? bytes_per_pixel(*params) : 0;
}

extern "C" int split_server_create(const split_server_config* cfg, split_server** out) {
  if (!cfg || !out) return SPLIT_ERR_INVALID;
  *out = nullptr;
  split_server_config c = *cfg;
  if (c.hbm_budget_bytes == 0) c.hbm_budget_bytes = kDefaultBudget;
  if (c.max_batch_pixels <= 0) c.max_batch_pixels = kDefaultMaxBatchPixels;
  if (c.max_inflight <= 0) c.max_inflight = 2;
  if (c.max_inflight > 8) return SPLIT_ERR_INVALID;
  split_batch_image probe{64, 64, 4, 1};
  split_batch* pb = nullptr;
  SG_TRY(split_batch_create(&probe, 1, &c.params, &pb));   // validates the parameters
  split_batch_destroy(pb);
  int prev = 0;
  SG_CUDA_TRY(cudaGetDevice(&prev));
  SG_CUDA_TRY(cudaSetDevice(c.device));
  split_server* s = new (std::nothrow) split_server();
  if (!s) return SPLIT_ERR_WORKSPACE;
  s->cfg = c;
  s->bpp = bytes_per_pixel(c.params);
  s->adm.budget = c.hbm_budget_bytes;
  s->slots.resize(c.max_inflight);
  int st = SPLIT_OK;
  if (cudaStreamCreateWithFlags(&s->h2d, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s->compute, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s->d2h, cudaStreamNonBlocking) != cudaSuccess || !s->bpp)
    st = SPLIT_ERR_CUDA;
  cudaSetDevice(prev);
  if (st != SPLIT_OK) {
    split_server_destroy(s);
    return st;
  }
  s->worker = std::thread(worker_main, s);
  *out = s;
  return SPLIT_OK;
}

extern "C" int split_server_reserve(split_server* s, int64_t pixels, int max_requests) {
  if (!s || pixels < 1 || max_requests < 1) return SPLIT_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->nflights > 0 || !s->adm.waiting.empty() || !s->adm.admitted.empty())
    return SPLIT_ERR_INVALID;   // only while the server is idle
  // a batch of `pixels` in one image, clustered more than once, gives the
  // workspace bound (its kept span sums, pixels / 128 spans, bound those of
  // any images of the same total); every image of a batch may add a
  // 64-pixel granule of arena
  const int side = 8192;
  split_batch_image im{side, (int)((pixels + side - 1) / side) + 2, 64, 2};
  split_batch* b = nullptr;
  SG_TRY(split_batch_create(&im, 1, &s->cfg.params, &b));
  const size_t wsb = split_batch_workspace_size(b);
  split_batch_destroy(b);
  int prev = 0;
  SG_CUDA_TRY(cudaGetDevice(&prev));
  SG_CUDA_TRY(cudaSetDevice(s->cfg.device));
  int st = SPLIT_OK;
  for (Slot& sl : s->slots) {
    st = sl.ensure(pixels + kGranule * max_requests, (int64_t)s->cfg.params.dim * 64 * max_requests,
                   wsb, s->cfg.params.compute_normals != 0, s->h2d);
    if (st != SPLIT_OK) break;
  }
  if (st == SPLIT_OK && cudaStreamSynchronize(s->h2d) != cudaSuccess) st = SPLIT_ERR_CUDA;
  cudaSetDevice(prev);
  return st;
}

extern "C" int split_server_submit(split_server* s, const split_request* r, uint64_t* ticket) {
  if (!s || !r || !r->rgb || !r->centroids || !r->segment_labels || r->width < 1 ||
      r->height < 1 || r->nclusters < 1 || r->nclusters > 64 || r->kmeans_iters < 0)
    return SPLIT_ERR_INVALID;
  if ((int64_t)r->width * r->height > 0x7fffffffLL / 3) return SPLIT_ERR_INVALID;
  Req q;
  q.r = *r;
  q.pixels = (int64_t)r->width * r->height;
  q.footprint = (size_t)rounded(q.pixels) * s->bpp;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return SPLIT_ERR_INVALID;
    if (q.footprint > s->adm.budget) return SPLIT_ERR_WORKSPACE;   // could never be admitted
    q.ticket = s->next_ticket++;
    q.submitted = Clock::now();
    s->adm.waiting.push_back(q);
    s->submitted += 1;
  }
  s->work_cv.notify_all();
  if (ticket) *ticket = q.ticket;
  return SPLIT_OK;
}

extern "C" int split_server_poll(split_server* s, split_completion* out, int max, int timeout_ms,
                                 int* n) {
  if (!s || !out || max < 1 || !n) return SPLIT_ERR_INVALID;
  *n = 0;
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->done.empty() && timeout_ms != 0) {
    auto ready = [&] { return !s->done.empty(); };
    if (timeout_ms < 0)
      s->done_cv.wait(lk, [&] { return ready() || s->completed == s->submitted; });
    else
      s->done_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready);
  }
  while (*n < max && !s->done.empty()) {
    out[(*n)++] = s->done.front();
    s->done.pop_front();
  }
  return SPLIT_OK;
}

extern "C" int split_server_stats(split_server* s, split_server_counters* out) {
  if (!s || !out) return SPLIT_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->mu);
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->batches = s->batches;
  out->in_use_bytes = s->adm.in_use;
  out->peak_in_use_bytes = s->adm.peak;
  out->bytes_per_pixel = s->bpp;
  out->budget_bytes = s->adm.budget;
  return SPLIT_OK;
}

extern "C" int split_server_destroy(split_server* s) {
  if (!s) return SPLIT_ERR_INVALID;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->work_cv.notify_all();
  if (s->worker.joinable()) s->worker.join();   // drains every submitted request
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(s->cfg.device);
  if (s->h2d) cudaStreamSynchronize(s->h2d);
  if (s->compute) cudaStreamSynchronize(s->compute);
  if (s->d2h) cudaStreamSynchronize(s->d2h);
  for (Slot& sl : s->slots) sl.free_all();
  if (s->h2d) cudaStreamDestroy(s->h2d);
  if (s->compute) cudaStreamDestroy(s->compute);
  if (s->d2h) cudaStreamDestroy(s->d2h);
  cudaSetDevice(prev);
  delete s;
  return SPLIT_OK;
}

// Host-side test of the admission and batch-formation policy (no GPU): all
// requests arrive at once, batches launch while fewer than `max_inflight`
// are outstanding, and the oldest batch completes whenever no further batch
// can launch.  batch_of[i] receives the batch index of request i; returns the
// number of batches, or a negative status.
extern "C" int split_server_admission_test(const int64_t* footprints, const int64_t* pixels,
                                           int n, int64_t budget, int64_t max_batch_pixels,
                                           int max_inflight, int32_t* batch_of,
                                           int64_t* peak_in_use) {
  if (!footprints || !pixels || !batch_of || n < 0 || budget < 0 || max_inflight < 1)
    return -SPLIT_ERR_INVALID;
  Admission a;
  a.budget = (size_t)budget;
  for (int i = 0; i < n; ++i) {
    if (footprints[i] < 0 || (size_t)footprints[i] > a.budget) return -SPLIT_ERR_WORKSPACE;
    Req q{};
    q.ticket = (uint64_t)i;
    q.pixels = pixels[i];
    q.footprint = (size_t)footprints[i];
    a.waiting.push_back(q);
  }
  std::deque<std::vector<Req>> inflight;
  int nb = 0, done = 0;
  while (done < n) {
    a.admit();
    if (!a.admitted.empty() && (int)inflight.size() < max_inflight) {
      std::vector<Req> b = a.take(max_batch_pixels);
      for (const Req& q : b) batch_of[q.ticket] = nb;
      ++nb;
      inflight.push_back(std::move(b));
      continue;
    }
    if (inflight.empty()) return -SPLIT_ERR_INVALID;   // cannot happen: the head always fits
    a.release(inflight.front());
    done += (int)inflight.front().size();
    inflight.pop_front();
  }
  if (peak_in_use) *peak_in_use = (int64_t)a.peak;
  return nb;
}
