// gst_server.cpp -- continuous-batching decode server (gst_server_* in
// include/gst_decoder.h).  No counterpart in the reference, whose demos decode
// fixed pages of pre-packed streams (demo/photos_sf.cpp:688-830).
//
// Requests are whole GST streams submitted from host memory.  A scheduler
// thread
//   * admits queued requests in arrival order while their compressed bytes and
//     DXT1 output fit in the device budget (first-fit over one device arena),
//   * launches whatever is admitted as one batch as soon as one of
//     `max_inflight` launch slots is free (each slot has its own stream, plan
//     buffers and scratch), so batches overlap on the device and requests that
//     arrive meanwhile ride in the next launch,
//   * retires a launch when a host function enqueued behind it runs: the
//     compressed input is freed at once, the DXT1 output stays resident until
//     the caller releases it.
// Every image keeps its own GST stream and output region: the plan carries
// absolute device addresses (write_plan with freq_at/body_at/out_at), so a batch
// needs no packing on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "gst_decoder.h"
#include "gst_host.h"
#include "gst_plan.h"

using namespace gst;
using namespace gst::host;

namespace {

using Clock = std::chrono::steady_clock;
constexpr size_t kGranule = 256;

// First-fit allocator over [0, size) in 256-byte granules, with coalescing.
class Arena {
 public:
  void reset(size_t size) {
    free_.clear();
    if (size) free_[0] = size;
    used_ = 0;
  }
  bool alloc(size_t bytes, size_t *off) {
    bytes = align_up(std::max<size_t>(bytes, 1), kGranule);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < bytes) continue;
      *off = it->first;
      const size_t rest = it->second - bytes, start = it->first + bytes;
      free_.erase(it);
      if (rest) free_[start] = rest;
      used_ += bytes;
      return true;
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = align_up(std::max<size_t>(bytes, 1), kGranule);
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  size_t used() const { return used_; }

 private:
  std::map<size_t, size_t> free_;
  size_t used_ = 0;
};

enum class State { kQueued, kAdmitted, kLaunched, kDone };

struct Request {
  uint64_t id = 0;
  gst_header hdr = {};
  size_t len = 0;
  size_t host_off = 0;
  size_t in_off = 0, out_off = 0;
  uint64_t t_arrival = 0, t_launch = 0, t_done = 0;  // ns on the server clock
  gst_status status = GST_OK;
  State state = State::kQueued;
};

struct Slot {
  cudaStream_t stream = nullptr;
  uint8_t *plan_h = nullptr, *plan_d = nullptr;
  size_t plan_cap = 0;
  uint8_t *scratch = nullptr;
  size_t scratch_cap = 0;
  uint32_t *status_d = nullptr;  // the launches' status word (per-image words are read instead)
  size_t err_off = 0;            // per-image error words in the plan, copied back into plan_h
  std::vector<uint64_t> ids;
  std::vector<gst_header> hdrs;
  std::vector<uint64_t> freq_at, body_at, out_at;
  bool busy = false;
  uint64_t t_done = 0;
  struct gst_server *srv = nullptr;
};

size_t dxt_bytes(const gst_header &h) { return size_t(image_blocks(h)) * 8; }

}  // namespace

struct gst_server {
  gst_ctx *ctx = nullptr;
  int device = 0;
  gst_server_config cfg = {};
  Clock::time_point t0;
  uint8_t *dev = nullptr;  // device arena: compressed inputs + DXT1 outputs
  uint8_t *host = nullptr; // pinned staging of submitted streams
  Arena dev_arena, host_arena;
  std::vector<Slot> slots;

  std::mutex mu;
  std::condition_variable cv;       // wakes the scheduler
  std::condition_variable done_cv;  // wakes pollers
  bool stop = false;
  bool failed = false;
  gst_status fail_status = GST_OK;
  uint64_t next_id = 1;
  std::unordered_map<uint64_t, Request> reqs;
  std::deque<uint64_t> queued, admitted, done;
  std::vector<Slot *> retired;  // slots whose host function has run
  std::thread thread;

  // statistics since the last reset
  // Completed requests' latencies: chunked storage, so that appending under
  // the lock never reallocates and copies the whole record (at 20k req/s a
  // vector's doubling copied megabytes while submissions waited).
  std::deque<double> lat_us;
  uint64_t submitted = 0, completed = 0, rejected = 0, cancelled = 0, launches = 0, launched_images = 0, pixels = 0;
  uint64_t t_stats = 0;
  size_t dev_peak = 0;

  // open-loop submissions from a native thread (gst_server_schedule); sched_mu
  // guards the thread object against concurrent schedule / schedule_wait calls
  std::mutex sched_mu;
  std::thread sched;
  std::atomic<bool> sched_stop{false};
  int sched_submitted = 0, sched_rejected = 0;
  uint64_t sched_late_max = 0;
  gst_status sched_status = GST_OK;

  uint64_t now() const {
    return uint64_t(std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - t0).count());
  }
  void run();
  bool launch(Slot &s, std::unique_lock<std::mutex> &lk);
};

namespace {

void CUDART_CB slot_done(void *p) {
  Slot *s = static_cast<Slot *>(p);
  gst_server *srv = s->srv;
  const uint64_t t = srv->now();
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    s->t_done = t;
    srv->retired.push_back(s);
  }
  srv->cv.notify_one();
}

gst_status grow(uint8_t **dev_p, uint8_t **host_p, size_t *cap, size_t need) {
  if (*cap >= need) return GST_OK;
  const size_t sz = std::max(need, *cap * 2);
  if (dev_p) {
    cudaFree(*dev_p);
    *dev_p = nullptr;
    cudaError_t e = cudaMalloc(reinterpret_cast<void **>(dev_p), sz);
    if (e != cudaSuccess) {
      *dev_p = nullptr;
      *cap = 0;
      return cuda_status(e);
    }
  }
  if (host_p) {
    cudaFreeHost(*host_p);
    *host_p = nullptr;
    cudaError_t e = cudaMallocHost(reinterpret_cast<void **>(host_p), sz);
    if (e != cudaSuccess) {
      *host_p = nullptr;
      *cap = 0;
      return cuda_status(e);
    }
  }
  *cap = sz;
  return GST_OK;
}

// Plan bytes of a launch of at most n images whose scratch totals at most
// `scratch` bytes: each image takes at least 8 bytes of scratch per block, so
// there are at most scratch / 8192 tiles and full rANS items (an item covers
// at least one 8192-symbol group), plus one partial item per section.
size_t plan_bytes_bound(size_t scratch, int n) {
  const size_t units = scratch / kSymsPerGroup;
  const size_t rans = units + 4 * size_t(n);
  return align_up(sizeof(GstPlanHead), 128) + sizeof(GstImageDesc) * size_t(n) + (sizeof(GstRansItem) + 4) * rans +
         sizeof(GstTileItem) * units + 12 * size_t(n) + 16 + 64;
}

}  // namespace

// Builds and enqueues one batch on slot s from the admitted queue.  Called
// with the lock held; drops it around the CUDA calls.  Returns false if
// nothing was launched.
bool gst_server::launch(Slot &s, std::unique_lock<std::mutex> &lk) {
  s.ids.clear();
  s.hdrs.clear();
  s.freq_at.clear();
  s.body_at.clear();
  s.out_at.clear();
  size_t scratch = 0;
  const int cap = cfg.max_batch_images;
  while (!admitted.empty() && int(s.ids.size()) < cap) {
    Request &r = reqs[admitted.front()];
    const size_t need = scratch_layout(r.hdr).total;
    if (!s.ids.empty() && scratch + need > cfg.slot_scratch_bytes) break;
    scratch += need;
    r.state = State::kLaunched;
    r.t_launch = now();
    s.ids.push_back(r.id);
    s.hdrs.push_back(r.hdr);
    s.freq_at.push_back(reinterpret_cast<uint64_t>(dev + r.in_off + 28));
    s.body_at.push_back(reinterpret_cast<uint64_t>(dev + r.in_off + 28 + 4 * kFreqTableBytes));
    s.out_at.push_back(reinterpret_cast<uint64_t>(dev + r.out_off));
    admitted.pop_front();
  }
  if (s.ids.empty()) return false;
  s.busy = true;
  std::vector<std::pair<size_t, std::pair<size_t, size_t>>> copies;  // (host_off, (dev_off, len))
  for (uint64_t id : s.ids) {
    const Request &r = reqs[id];
    copies.push_back({r.host_off, {r.in_off, r.len}});
  }
  lk.unlock();

  const int n = int(s.ids.size());
  NvtxRange range("gst server launch");
  GstTuning tuning = ctx_tuning_for(ctx, s.hdrs.data(), n);
  tuning.persistent = 0;
  const PlanLayout L = plan_layout(s.hdrs.data(), n, plan_capacity(ctx, tuning));
  gst_status st = grow(&s.scratch, nullptr, &s.scratch_cap, L.scratch_bytes);
  if (st == GST_OK && s.plan_cap < L.bytes) {
    cudaFree(s.plan_d);
    s.plan_d = nullptr;
    size_t c = 0;
    st = grow(&s.plan_d, nullptr, &c, L.bytes);
    if (st == GST_OK) {
      cudaFreeHost(s.plan_h);
      s.plan_h = nullptr;
      size_t c2 = 0;
      st = grow(nullptr, &s.plan_h, &c2, L.bytes);
      s.plan_cap = std::min(c, c2);
    }
  }
  cudaError_t e = cudaSuccess;
  if (st == GST_OK) {
    write_plan(L, s.hdrs.data(), n, s.plan_h, s.freq_at.data(), s.body_at.data(), s.out_at.data());
    for (auto &c : copies) {
      e = cudaMemcpyAsync(dev + c.second.first, host + c.first, c.second.second, cudaMemcpyHostToDevice, s.stream);
      if (e != cudaSuccess) break;
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(s.plan_d, s.plan_h, L.bytes, cudaMemcpyHostToDevice, s.stream);
    int nl = 0;
    // The launch's size class gives CTAs per SM and staging depth; launches
    // on different slots run side by side, so the two-kernel form is kept
    // (a persistent launch fills every SM and would hold the others back).
    if (e == cudaSuccess)
      e = launch_decode(nullptr, s.scratch, nullptr, plan_view(L, s.plan_d, s.status_d), s.stream, &nl, nullptr,
                        tuning);
    // Per-image error words back into the pinned plan copy, then retire.
    s.err_off = L.off_image_err;
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(s.plan_h + L.off_image_err, s.plan_d + L.off_image_err, 4 * size_t(n),
                          cudaMemcpyDeviceToHost, s.stream);
    if (e == cudaSuccess) e = cudaLaunchHostFunc(s.stream, slot_done, &s);
    if (e != cudaSuccess) st = cuda_status(e);
  }
  lk.lock();
  ++launches;
  launched_images += uint64_t(n);
  if (st != GST_OK) {
    // Nothing will retire this slot: fail the server (the stream may hold
    // enqueued work, so the slot is not reused).
    failed = true;
    fail_status = st;
  }
  return true;
}

void gst_server::run() {
  cudaSetDevice(device);
  std::unique_lock<std::mutex> lk(mu);
  for (;;) {
    bool progress = false;
    // 1. Retire finished launches.
    for (Slot *s : retired) {
      const uint32_t *image_err = reinterpret_cast<const uint32_t *>(s->plan_h + s->err_off);
      for (size_t k = 0; k < s->ids.size(); ++k) {
        Request &r = reqs[s->ids[k]];
        r.t_done = s->t_done;
        r.status = image_err[k] ? GST_E_FORMAT : GST_OK;
        r.state = State::kDone;
        dev_arena.release(r.in_off, r.len);
        host_arena.release(r.host_off, r.len);
        lat_us.push_back(double(r.t_done - r.t_arrival) / 1e3);
        pixels += uint64_t(r.hdr.width) * r.hdr.height;
        ++completed;
        done.push_back(r.id);
      }
      s->busy = false;
      progress = true;
    }
    if (!retired.empty()) done_cv.notify_all();
    retired.clear();
    // 2. Admit in arrival order while the budget holds.
    while (!queued.empty()) {
      Request &r = reqs[queued.front()];
      size_t in_off = 0, out_off = 0;
      if (!dev_arena.alloc(r.len, &in_off)) break;
      if (!dev_arena.alloc(dxt_bytes(r.hdr), &out_off)) {
        dev_arena.release(in_off, r.len);
        break;
      }
      r.in_off = in_off;
      r.out_off = out_off;
      r.state = State::kAdmitted;
      admitted.push_back(r.id);
      queued.pop_front();
      dev_peak = std::max(dev_peak, dev_arena.used());
      progress = true;
    }
    // 3. Launch into free slots.
    if (!failed) {
      for (Slot &s : slots) {
        if (admitted.empty()) break;
        if (s.busy) continue;
        if (launch(s, lk)) progress = true;
        if (failed) break;
      }
    }
    if (failed) done_cv.notify_all();
    bool idle = true;
    for (const Slot &s : slots) idle = idle && !s.busy;
    if (stop && idle) break;  // requests not yet launched are dropped
    if (!progress) cv.wait_for(lk, std::chrono::microseconds(200));
  }
}

extern "C" {

gst_status gst_server_create(gst_ctx *ctx, const gst_server_config *cfg, gst_server **out) {
  if (!ctx || !out) return GST_E_ARG;
  *out = nullptr;
  gst_server_config c = {};
  if (cfg) c = *cfg;
  if (!c.device_budget_bytes) c.device_budget_bytes = size_t(32) << 30;
  if (!c.host_staging_bytes) c.host_staging_bytes = size_t(1) << 30;
  if (c.max_inflight <= 0) c.max_inflight = 4;
  if (c.max_batch_images <= 0) c.max_batch_images = 256;
  if (!c.slot_scratch_bytes) c.slot_scratch_bytes = size_t(256) << 20;
  if (c.max_inflight > 64) return GST_E_ARG;

  gst_server *srv = new gst_server();
  srv->ctx = ctx;
  srv->device = ctx_device(ctx);
  srv->cfg = c;
  srv->t0 = Clock::now();
  cudaSetDevice(srv->device);
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(&srv->dev), c.device_budget_bytes);
  if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void **>(&srv->host), c.host_staging_bytes);
  srv->slots.resize(size_t(c.max_inflight));
  for (Slot &s : srv->slots) {
    s.srv = srv;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void **>(&s.status_d), sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemset(s.status_d, 0, sizeof(uint32_t));
    // Scratch and plan buffers are sized up front for a full launch (the
    // admission rule keeps a launch's scratch within slot_scratch_bytes), so
    // no allocation (cudaFree synchronises the device) happens while serving;
    // only a single image above the limit grows them.
    if (e == cudaSuccess) {
      gst_status st = grow(&s.scratch, nullptr, &s.scratch_cap, c.slot_scratch_bytes);
      const size_t pb = plan_bytes_bound(c.slot_scratch_bytes, c.max_batch_images);
      size_t c1 = 0, c2 = 0;
      if (st == GST_OK) st = grow(&s.plan_d, nullptr, &c1, pb);
      if (st == GST_OK) st = grow(nullptr, &s.plan_h, &c2, pb);
      s.plan_cap = std::min(c1, c2);
      if (st != GST_OK) e = cudaErrorMemoryAllocation;
    }
  }
  if (e != cudaSuccess) {
    gst_server_destroy(srv);
    return cuda_status(e);
  }
  srv->dev_arena.reset(c.device_budget_bytes);
  srv->host_arena.reset(c.host_staging_bytes);
  srv->thread = std::thread([srv] { srv->run(); });
  *out = srv;
  return GST_OK;
}

void gst_server_destroy(gst_server *srv) {
  if (!srv) return;
  {
    std::lock_guard<std::mutex> sl(srv->sched_mu);
    if (srv->sched.joinable()) {
      srv->sched_stop = true;
      srv->sched.join();
    }
  }
  if (srv->thread.joinable()) {
    {
      std::lock_guard<std::mutex> lk(srv->mu);
      srv->stop = true;
    }
    srv->cv.notify_one();
    srv->thread.join();
  }
  cudaSetDevice(srv->device);
  for (Slot &s : srv->slots) {
    if (s.stream) cudaStreamSynchronize(s.stream);
  }
  for (Slot &s : srv->slots) {
    if (s.stream) cudaStreamDestroy(s.stream);
    cudaFree(s.plan_d);
    cudaFreeHost(s.plan_h);
    cudaFree(s.scratch);
    cudaFree(s.status_d);
  }
  cudaFree(srv->dev);
  cudaFreeHost(srv->host);
  delete srv;
}

uint64_t gst_server_now_ns(gst_server *srv) { return srv ? srv->now() : 0; }

gst_status gst_server_submit(gst_server *srv, const void *gst, size_t len, uint64_t arrival_ns, uint64_t *id) {
  if (!srv || !gst || !id) return GST_E_ARG;
  gst_header h;
  gst_status st = gst_parse_header(static_cast<const uint8_t *>(gst), len, &h);
  if (st != GST_OK) return st;
  const size_t used = 28 + 4 * kFreqTableBytes + size_t(section_bytes(h));
  if (used + dxt_bytes(h) + 2 * kGranule > srv->cfg.device_budget_bytes) return GST_E_OOM;  // never admissible
  size_t host_off = 0;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    if (srv->failed) return srv->fail_status;
    if (!srv->host_arena.alloc(used, &host_off)) {
      ++srv->rejected;
      return GST_E_OOM;  // staging full: the caller may retry later
    }
  }
  memcpy(srv->host + host_off, gst, used);
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    Request r;
    r.id = srv->next_id++;
    r.hdr = h;
    r.len = used;
    r.host_off = host_off;
    r.t_arrival = arrival_ns ? arrival_ns : srv->now();
    *id = r.id;
    srv->reqs.emplace(r.id, r);
    srv->queued.push_back(r.id);
    ++srv->submitted;
  }
  srv->cv.notify_one();
  return GST_OK;
}

gst_status gst_server_schedule(gst_server *srv, int n, const void *const *gst, const size_t *len,
                               const uint64_t *arrival_ns, uint64_t *ids) {
  if (!srv || n < 0 || (n > 0 && (!gst || !len || !arrival_ns || !ids))) return GST_E_ARG;
  std::lock_guard<std::mutex> sl(srv->sched_mu);
  if (srv->sched.joinable()) return GST_E_ARG;  // one schedule at a time: wait for the last one first
  srv->sched_stop = false;
  srv->sched = std::thread([srv, n, gst, len, arrival_ns, ids] {
    int sub = 0, rej = 0;
    uint64_t late = 0;
    gst_status status = GST_OK;
    int i = 0;
    for (; i < n && !srv->sched_stop; ++i) {
      const uint64_t at = arrival_ns[i];
      // Sleep through long gaps, spin through short ones: yielding the core
      // can cost a whole scheduler time slice (measured: submissions up to
      // 30 ms late at 20k req/s).
      for (uint64_t t = srv->now(); t < at && !srv->sched_stop; t = srv->now()) {
        const uint64_t ahead = at - t;
        if (ahead > 250000) std::this_thread::sleep_for(std::chrono::nanoseconds(ahead - 150000));
      }
      const uint64_t t = srv->now();
      late = std::max(late, t > at ? t - at : uint64_t(0));
      // the id is written under the server's lock, before the request can run
      const gst_status st = gst_server_submit(srv, gst[i], len[i], at, &ids[i]);
      if (st == GST_OK) {
        ++sub;
      } else if (st == GST_E_OOM) {
        ids[i] = 0;  // staging full at its arrival, or never admissible
        ++rej;
      } else {
        status = st;
        break;
      }
    }
    for (; i < n; ++i) ids[i] = 0;
    std::lock_guard<std::mutex> lk(srv->mu);
    srv->sched_submitted = sub;
    srv->sched_rejected = rej;
    srv->sched_late_max = late;
    srv->sched_status = status;
  });
  return GST_OK;
}

gst_status gst_server_schedule_wait(gst_server *srv, int *submitted, int *rejected, uint64_t *late_max_ns) {
  if (!srv) return GST_E_ARG;
  std::lock_guard<std::mutex> sl(srv->sched_mu);
  if (!srv->sched.joinable()) return GST_E_ARG;
  srv->sched.join();
  std::lock_guard<std::mutex> lk(srv->mu);
  if (submitted) *submitted = srv->sched_submitted;
  if (rejected) *rejected = srv->sched_rejected;
  if (late_max_ns) *late_max_ns = srv->sched_late_max;
  return srv->sched_status;
}

gst_status gst_server_poll(gst_server *srv, gst_server_result *out, int cap, int *n, int wait_us) {
  if (!srv || !n || cap < 0 || (cap > 0 && !out)) return GST_E_ARG;
  *n = 0;
  std::unique_lock<std::mutex> lk(srv->mu);
  if (srv->done.empty() && wait_us > 0 && !srv->failed)
    srv->done_cv.wait_for(lk, std::chrono::microseconds(wait_us), [srv] { return !srv->done.empty() || srv->failed; });
  while (*n < cap && !srv->done.empty()) {
    const Request &r = srv->reqs[srv->done.front()];
    srv->done.pop_front();
    gst_server_result &o = out[(*n)++];
    o.id = r.id;
    o.status = r.status;
    o.d_dxt = srv->dev + r.out_off;
    o.dxt_bytes = dxt_bytes(r.hdr);
    o.width = r.hdr.width;
    o.height = r.hdr.height;
    o.arrival_ns = r.t_arrival;
    o.launch_ns = r.t_launch;
    o.done_ns = r.t_done;
  }
  if (*n == 0 && srv->failed) return srv->fail_status;
  return GST_OK;
}

gst_status gst_server_read(gst_server *srv, uint64_t id, void *dst, size_t cap) {
  if (!srv || !dst) return GST_E_ARG;
  size_t off = 0, bytes = 0;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(id);
    if (it == srv->reqs.end() || it->second.state != State::kDone) return GST_E_ARG;
    off = it->second.out_off;
    bytes = dxt_bytes(it->second.hdr);
  }
  if (cap < bytes) return GST_E_ARG;
  cudaSetDevice(srv->device);
  return cuda_status(cudaMemcpy(dst, srv->dev + off, bytes, cudaMemcpyDeviceToHost));
}

gst_status gst_server_release(gst_server *srv, uint64_t id) {
  if (!srv) return GST_E_ARG;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(id);
    if (it == srv->reqs.end() || it->second.state != State::kDone) return GST_E_ARG;
    srv->dev_arena.release(it->second.out_off, dxt_bytes(it->second.hdr));
    srv->reqs.erase(it);
  }
  srv->cv.notify_one();  // memory freed: the scheduler may admit more
  return GST_OK;
}

gst_status gst_server_cancel(gst_server *srv, uint64_t id) {
  if (!srv) return GST_E_ARG;
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(id);
    if (it == srv->reqs.end()) return GST_E_ARG;
    Request &r = it->second;
    std::deque<uint64_t> *q = nullptr;
    if (r.state == State::kQueued) q = &srv->queued;
    else if (r.state == State::kAdmitted) q = &srv->admitted;
    else return GST_E_ARG;  // launched or done: it completes normally
    auto pos = std::find(q->begin(), q->end(), id);
    if (pos == q->end()) return GST_E_ARG;
    q->erase(pos);
    if (r.state == State::kAdmitted) {
      srv->dev_arena.release(r.in_off, r.len);
      srv->dev_arena.release(r.out_off, dxt_bytes(r.hdr));
    }
    srv->host_arena.release(r.host_off, r.len);
    srv->reqs.erase(it);
    ++srv->cancelled;
  }
  srv->cv.notify_one();  // staging or budget freed: the scheduler may admit more
  return GST_OK;
}

gst_status gst_server_read_stats(gst_server *srv, gst_server_stats *st, int reset) {
  if (!srv || !st) return GST_E_ARG;
  std::vector<double> v;  // the latencies, sorted outside the lock
  {
    std::lock_guard<std::mutex> lk(srv->mu);
    memset(st, 0, sizeof(*st));
    st->submitted = srv->submitted;
    st->completed = srv->completed;
    st->rejected = srv->rejected;
    st->cancelled = srv->cancelled;
    st->launches = srv->launches;
    st->launched_images = srv->launched_images;
    st->pixels = srv->pixels;
    st->queued = srv->queued.size();
    st->device_bytes_in_use = srv->dev_arena.used();
    st->device_bytes_peak = srv->dev_peak;
    const uint64_t t = srv->now();
    st->seconds = double(t - srv->t_stats) / 1e9;
    v.assign(srv->lat_us.begin(), srv->lat_us.end());
    if (reset) {
      srv->lat_us.clear();
      srv->submitted = srv->completed = srv->rejected = srv->cancelled = srv->launches = srv->launched_images =
          srv->pixels = 0;
      srv->dev_peak = srv->dev_arena.used();
      srv->t_stats = t;
    }
  }
  if (!v.empty()) {
    std::sort(v.begin(), v.end());
    auto pct = [&](double p) {
      const size_t k = std::min(v.size() - 1, size_t(p / 100.0 * double(v.size() - 1) + 0.5));
      return v[k];
    };
    double sum = 0;
    for (double x : v) sum += x;
    st->latency_mean_us = sum / double(v.size());
    st->latency_p50_us = pct(50);
    st->latency_p99_us = pct(99);
    st->latency_max_us = v.back();
  }
  return GST_OK;
}

}  // extern "C"
