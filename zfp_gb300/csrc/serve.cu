// serve.cu -- continuous batching of compress / decompress requests.
//
// The reference serves nothing; a caller of zfp_compress waits for each
// field in turn.  Here a dispatcher thread owns a few CUDA streams ("lanes").
// Requests are sorted by raw size into classes (up to 2 MiB, up to 32 MiB,
// larger), each with its own FIFO and its own lanes, so a small request
// never shares a launch with -- and never completes with -- a large one.
// Whenever a lane is free the dispatcher takes requests from the front of
// its class's FIFO while the bytes held by all admitted, unfinished requests
// stay within the HBM budget, and launches them as one batch: jobs grouped
// by (direction, type, dims), one persistent multi-job launch per group (the
// same kernels as zfp_compress).  A host callback at the end of the lane's
// work marks the batch complete and wakes the dispatcher, which publishes
// the results, returns the budget and admits whatever arrived in the
// meantime -- new work starts while other lanes are still running.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include "../../include/zfp_gb300.h"
#include "gpu_internal.h"
#include "runtime.h"

namespace zg {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t ticket = 0;
  int direction = 0;
  zfp_stream* z = nullptr;
  FieldInfo fi;
  Job job;
  size_t cost = 0;               // bytes counted against the budget
  int cls = 0;                   // size class (of the lanes that serve it)
  bool fixed = false;
  uint64_t nominal_end = 0;
  IndexRef held;                 // decompress: the block index read (kept until the request is gone)
  Clock::time_point t_submit, t_done;
  bool done = false;
  size_t size = 0;
};

// request size classes: raw bytes up to these bounds, then the rest
constexpr size_t kClassBound[] = {size_t(2) << 20, size_t(32) << 20};
constexpr int kClasses = 3;

static int size_class(size_t raw) {
  int c = 0;
  while (c < kClasses - 1 && raw > kClassBound[c]) c++;
  return c;
}

struct Lane {
  int cls = 0;                   // the size class it serves
  cudaStream_t st = nullptr;
  bool busy = false;
  std::atomic<bool> finished{false};
  std::vector<std::shared_ptr<Request>> reqs;
  void* dev = nullptr;           // jobs, scratch, results, index of the running batch
  JobResult* host_results = nullptr;   // pinned
  Job* host_jobs = nullptr;      // pinned staging for the job arrays
  size_t host_jobs_cap = 0;
  // outgrown staging buffers, freed with the server: cudaFreeHost waits for
  // the whole device, which would stall every lane in the middle of serving
  std::vector<void*> retired;
  std::vector<size_t> index_off; // per request: offset of its block index in `dev` (compress, variable rate)
  struct Server* server = nullptr;
};

struct Server {
  size_t budget = 0, used = 0;
  size_t peak = 0;               // most bytes ever admitted at once
  uint64_t batches = 0, served = 0;
  std::vector<std::unique_ptr<Lane>> lanes;
  std::deque<std::shared_ptr<Request>> pending[kClasses];   // per size class (lanes serve the classes they map to)
  int lane_class_max = 0;
  std::unordered_map<uint64_t, std::shared_ptr<Request>> live;
  std::mutex mu;
  std::condition_variable cv;
  std::thread worker;
  bool stop = false;
  uint64_t next_ticket = 1;
  int device = 0;
};

// pinned staging for `cap` jobs and results; the old buffers are retired
// (freed with the server), not freed now
static cudaError_t grow_staging(Lane* lane, size_t cap) {
  Job* jobs = nullptr;
  JobResult* results = nullptr;
  cudaError_t e = cudaHostAlloc((void**)&jobs, cap * sizeof(Job), 0);
  if (e != cudaSuccess) return e;
  if ((e = cudaHostAlloc((void**)&results, cap * sizeof(JobResult), 0)) != cudaSuccess) {
    lane->retired.push_back(jobs);
    return e;
  }
  if (lane->host_jobs) lane->retired.push_back(lane->host_jobs);
  if (lane->host_results) lane->retired.push_back(lane->host_results);
  lane->host_jobs = jobs;
  lane->host_results = results;
  lane->host_jobs_cap = cap;
  return cudaSuccess;
}

static void CUDART_CB lane_done(void* arg) {
  Lane* lane = (Lane*)arg;
  const Clock::time_point now = Clock::now();
  {
    std::lock_guard<std::mutex> lk(lane->server->mu);
    for (auto& r : lane->reqs) r->t_done = now;
    lane->finished = true;
  }
  lane->server->cv.notify_all();
}

// launch the lane's requests; called without the server lock
static cudaError_t launch_batch(Server* s, Lane* lane) {
  auto& reqs = lane->reqs;
  // group by (direction, type, dims) -- one launch each -- and assign tiles
  std::map<std::tuple<int, int, int, bool>, std::vector<size_t>> groups;
  for (size_t i = 0; i < reqs.size(); i++)
    groups[{reqs[i]->direction, reqs[i]->fi.type, reqs[i]->fi.dims, reqs[i]->z->minexp < ZFP_MIN_EXP}].push_back(i);
  // device layout: results | per group: jobs, scratch | block indexes
  size_t off = ((reqs.size() * sizeof(JobResult)) + 255) & ~(size_t)255;
  struct G { int type, dims; bool lossy; std::vector<size_t> idx; uint32_t tiles = 0, img_words = 0; size_t jobs_off,
             scr_off, scr_bytes; LaunchArgs one; };
  std::vector<G> gs;
  for (auto& kv : groups) {
    G g;
    g.type = std::get<1>(kv.first);
    g.dims = std::get<2>(kv.first);
    g.lossy = !std::get<3>(kv.first);
    g.idx = kv.second;
    for (size_t i : g.idx) {
      Request& r = *reqs[i];
      r.job.tile0 = g.tiles;
      g.tiles += r.job.ntiles;
      const uint64_t bound = r.fixed ? (uint64_t)r.z->maxbits : block_bound(r.fi, r.z);
      g.img_words = std::max<uint32_t>(g.img_words, (uint32_t)image_words((uint64_t)kTile * bound / 64 + 4));
    }
    g.jobs_off = off;
    off += ((g.idx.size() * sizeof(Job)) + 255) & ~(size_t)255;
    const size_t t = (size_t)g.tiles + 1;
    g.scr_off = off;
    g.scr_bytes = 64 + t * 28;
    off += (g.scr_bytes + 255) & ~(size_t)255;
    // a request alone in its group runs the kernel zfp_compress /
    // zfp_decompress would pick for it (specialised to its mode and sized
    // to it), planned the same way; several share the multi-job kernel
    std::memset(&g.one, 0, sizeof g.one);
    if (g.idx.size() == 1) {
      const Request& r = *reqs[g.idx[0]];
      LaunchArgs& a = g.one;
      a.one = r.job;
      a.njobs = 1;
      a.total_tiles = g.tiles;
      a.grid = (int)g.tiles;
      a.use_ticket = r.direction == 0 && !r.fixed;
      if (r.direction == 1 && g.tiles) {
        const uint64_t end = r.fixed ? r.nominal_end : r.job.end_bit;
        a.want_words = (uint32_t)std::min<uint64_t>(image_words((end - r.job.bit0) / g.tiles / 64 + 4), 1u << 30);
      }
      const bool fixed_encode = r.direction == 0 && r.fixed;   // places known without the look-back
      const uint32_t room = fixed_encode ? 0 : stage_room_any(g.type, g.dims, a, r.direction == 0);
      a.img_words = std::min(g.img_words, room);
    }
    gs.push_back(g);
  }
  lane->index_off.assign(reqs.size(), SIZE_MAX);
  for (size_t i = 0; i < reqs.size(); i++)
    if (reqs[i]->direction == 0 && !reqs[i]->fixed) {
      lane->index_off[i] = off;
      off += reqs[i]->fi.nblocks * 8;
    }
  cudaError_t e = cudaMallocAsync(&lane->dev, off, lane->st);
  if (e != cudaSuccess) return e;
  char* base = (char*)lane->dev;
  if ((e = cudaMemsetAsync(base, 0, reqs.size() * sizeof(JobResult), lane->st)) != cudaSuccess) return e;
  // host staging for job arrays and results
  size_t njobs = reqs.size();
  if (lane->host_jobs_cap < njobs) {
    if ((e = grow_staging(lane, std::max<size_t>(njobs, 2 * lane->host_jobs_cap))) != cudaSuccess) return e;
  }
  size_t hj = 0;
  for (auto& g : gs) {
    Job* first = lane->host_jobs + hj;
    for (size_t i : g.idx) {
      Request& r = *reqs[i];
      r.job.result = (JobResult*)base + i;
      if (lane->index_off[i] != SIZE_MAX) r.job.offsets = (uint64_t*)(base + lane->index_off[i]);
      lane->host_jobs[hj++] = r.job;
    }
    if ((e = cudaMemcpyAsync(base + g.jobs_off, first, g.idx.size() * sizeof(Job), cudaMemcpyHostToDevice,
                             lane->st)) != cudaSuccess ||
        (e = cudaMemsetAsync(base + g.scr_off, 0, g.scr_bytes, lane->st)) != cudaSuccess)
      return e;
    const Request& r0 = *reqs[g.idx[0]];
    const bool single = g.idx.size() == 1;
    LaunchArgs a;
    if (single) {
      a = g.one;
      a.one = lane->host_jobs[hj - 1];   // with its result and index pointers
    } else {
      std::memset(&a, 0, sizeof a);
      a.one = r0.job;
      a.jobs = (const Job*)(base + g.jobs_off);
      a.njobs = (int)g.idx.size();
      a.multi_lossy = g.lossy;
    }
    const size_t t = (size_t)g.tiles + 1;
    char* p = base + g.scr_off;
    a.sc.ticket = (unsigned int*)(p + 32);
    a.sc.tile_state = (unsigned long long*)(p + 64);
    a.sc.side = (unsigned long long*)(p + 64 + t * 8);
    a.sc.side_cnt = (unsigned int*)(p + 64 + t * 24);
    a.sc.wait_cycles = wait_cycles();
    a.total_tiles = g.tiles;
    const bool enc = reqs[g.idx[0]]->direction == 0;
    if (!single) {
      a.use_ticket = 1;
      // tiles larger than the kernel's occupancy room are coded straight
      // into the stream (encode) or read from it directly (decode)
      a.img_words = std::min(g.img_words, stage_room_any(g.type, g.dims, a, enc));
      a.grid = (int)std::min<uint64_t>(g.tiles, (uint64_t)persistent_grid());
    }
    e = enc ? launch_encode_any(g.type, g.dims, a, lane->st) : launch_decode_any(g.type, g.dims, a, lane->st);
    if (e != cudaSuccess) return e;
  }
  if ((e = cudaMemcpyAsync(lane->host_results, base, reqs.size() * sizeof(JobResult), cudaMemcpyDeviceToHost,
                           lane->st)) != cudaSuccess)
    return e;
  return cudaLaunchHostFunc(lane->st, lane_done, lane);
}

// publish a finished lane's results; called with the server lock held
static void finish_lane(Server* s, Lane* lane) {
  for (size_t i = 0; i < lane->reqs.size(); i++) {
    Request& r = *lane->reqs[i];
    const JobResult& res = lane->host_results[i];
    uint64_t end = 0;
    bool ok = res.status == 0;
    if (ok) {
      if (r.direction == 0) {
        end = r.fixed ? r.nominal_end : res.end_bit;
        const StreamState ss = get_stream_state(r.z->stream);
        if (!r.fixed) {  // keep the block index for later decompression of this stream
          cudaError_t ie;
          IndexRef idx = make_index(r.fi.nblocks, lane->st, ie);
          if (idx &&
              cudaMemcpyAsync(idx->ptr, (char*)lane->dev + lane->index_off[i], r.fi.nblocks * 8,
                              cudaMemcpyDeviceToDevice, lane->st) == cudaSuccess &&
              cudaEventCreateWithFlags(&idx->written, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventRecord(idx->written, lane->st) == cudaSuccess)
            registry_insert(make_entry(ss.begin, r.job.bit0, end, r.fi, r.job, idx));
          else
            cudaGetLastError();
        } else {
          registry_invalidate(ss.begin, r.job.bit0, end);
        }
      } else {
        end = r.fixed ? r.nominal_end : r.job.end_bit;
      }
      set_stream_flushed(r.z->stream, end);
      r.size = (size_t)((end + 63) / 64) * 8;
    }
    r.done = true;
    s->used -= r.cost;
    s->served++;
  }
  cudaFreeAsync(lane->dev, lane->st);
  lane->dev = nullptr;
  lane->reqs.clear();
  lane->busy = false;
  lane->finished = false;
}

static void dispatcher(Server* s) {
  cudaSetDevice(s->device);
  const size_t kMaxBatch = 4096;
  std::unique_lock<std::mutex> lk(s->mu);
  auto admissible = [&](const Lane& l) {
    const auto& q = s->pending[l.cls];
    return !l.busy && !q.empty() && s->used + q.front()->cost <= s->budget;
  };
  for (;;) {
    s->cv.wait(lk, [&] {
      if (s->stop) return true;
      for (auto& l : s->lanes)
        if ((l->busy && l->finished) || admissible(*l)) return true;
      return false;
    });
    bool any = false;
    for (auto& l : s->lanes)
      if (l->busy && l->finished) {
        finish_lane(s, l.get());
        any = true;
      }
    if (any) s->cv.notify_all();
    for (auto& l : s->lanes) {
      if (l->busy) continue;
      auto& q = s->pending[l->cls];
      while (!q.empty() && l->reqs.size() < kMaxBatch && s->used + q.front()->cost <= s->budget) {
        s->used += q.front()->cost;
        l->reqs.push_back(q.front());
        q.pop_front();
      }
      if (l->reqs.empty()) continue;
      s->peak = std::max(s->peak, s->used);
      s->batches++;
      l->busy = true;
      Lane* lane = l.get();
      lk.unlock();
      const cudaError_t e = launch_batch(s, lane);
      lk.lock();
      if (e != cudaSuccess) {  // fail the whole batch
        cudaGetLastError();
        for (auto& r : lane->reqs) {
          r->done = true;
          r->size = 0;
          r->t_done = Clock::now();
          s->used -= r->cost;
        }
        if (lane->dev) cudaFreeAsync(lane->dev, lane->st);
        lane->dev = nullptr;
        lane->reqs.clear();
        lane->busy = false;
        s->cv.notify_all();
      }
    }
    if (s->stop) {
      bool idle = true;
      for (auto& q : s->pending) idle &= q.empty();
      for (auto& l : s->lanes) idle &= !l->busy;
      if (idle) break;
    }
  }
}

}  // namespace zg

struct zfp_gb300_server : zg::Server {};

extern "C" {

zfp_gb300_server* zfp_gb300_server_create(size_t hbm_budget, int lanes) {
  using namespace zg;
  if (!hbm_budget || lanes < 1 || lanes > 32) {
    fail("zfp_gb300_server_create: bad arguments");
    return nullptr;
  }
  init_pool_once();
  zfp_gb300_server* s = new zfp_gb300_server();
  s->budget = hbm_budget;
  cudaGetDevice(&s->device);
  for (int i = 0; i < lanes; i++) {
    auto l = std::make_unique<Lane>();
    l->server = s;
    // one lane per class first (small, medium, large), the rest to the large class
    l->cls = std::min(i, kClasses - 1);
    s->lane_class_max = std::max(s->lane_class_max, l->cls);
    if (cudaStreamCreateWithFlags(&l->st, cudaStreamNonBlocking) != cudaSuccess) {
      fail("zfp_gb300_server_create: cannot create CUDA streams");
      for (auto& x : s->lanes) cudaStreamDestroy(x->st);
      delete s;
      return nullptr;
    }
    // staging for batches of up to 1024 requests, allocated now rather than
    // while serving (a failure here is retried when a batch needs it)
    if (grow_staging(l.get(), 1024) != cudaSuccess) cudaGetLastError();
    s->lanes.push_back(std::move(l));
  }
  s->worker = std::thread(dispatcher, s);
  return s;
}

uint64_t zfp_gb300_server_submit(zfp_gb300_server* s, zfp_stream* z, const zfp_field* f, int direction) {
  using namespace zg;
  if (!s || !z || !z->stream || !f || (direction != 0 && direction != 1)) {
    fail("zfp_gb300_server_submit: bad arguments");
    return 0;
  }
  auto r = std::make_shared<Request>();
  r->direction = direction;
  r->z = z;
  if (const char* why = field_info(f, r->fi)) {
    fail(why);
    return 0;
  }
  const StreamState ss = get_stream_state(z->stream);
  if (!ss.begin || !is_device_ptr(ss.begin) || !is_device_ptr(f->data)) {
    fail("zfp_gb300_server_submit: field and stream must be in device memory");
    return 0;
  }
  const FieldInfo& fi = r->fi;
  r->fixed = is_fixed_rate(fi, z);
  Job j = base_job(fi, z, f->data);
  j.flags = (r->fixed ? kFixedRate : 0u) | vector_flags(fi, f->data);
  j.words = ss.begin;
  j.cap_words = (uint64_t)(ss.end - ss.begin);
  if (direction == 0) {
    j.bit0 = (uint64_t)(ss.ptr - ss.begin) * 64 + ss.bits;
    j.head_word = ss.bits ? (ss.buffer & ((1ull << ss.bits) - 1)) : 0;
    if (!r->fixed) j.flags |= kWriteIndex;
  } else {
    j.bit0 = (uint64_t)(ss.ptr - ss.begin) * 64 - ss.bits;
    if (!r->fixed) {
      IndexEntry ent;
      if (registry_find(ss.begin, j.bit0, fi, z, ent)) {
        j.offsets = ent.index->ptr;
        j.end_bit = ent.end_bit;
        j.flags |= kVerify;
        r->held = ent.index;
      } else {
        fail("zfp_gb300_server_submit: variable-rate stream without a block index (use zfp_decompress)");
        return 0;
      }
    }
  }
  if (r->fixed) r->nominal_end = j.bit0 + fi.nblocks * (uint64_t)z->maxbits;
  if (r->fixed && (r->nominal_end + 63) / 64 > j.cap_words) {
    fail("zfp_gb300_server_submit: stream buffer too small");
    return 0;
  }
  r->job = j;
  r->cost = (size_t)(fi.hi - fi.lo + 1) * fi.esize + (size_t)j.cap_words * 8;
  if (r->cost > s->budget) {
    fail("zfp_gb300_server_submit: request larger than the HBM budget");
    return 0;
  }
  // a class without a lane of its own goes to the largest class that has one
  r->cls = std::min(size_class((size_t)(fi.hi - fi.lo + 1) * fi.esize), s->lane_class_max);
  r->t_submit = Clock::now();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r->ticket = s->next_ticket++;
    s->live[r->ticket] = r;
    s->pending[r->cls].push_back(r);
  }
  s->cv.notify_all();
  return r->ticket;
}

size_t zfp_gb300_server_wait(zfp_gb300_server* s, uint64_t ticket, double* seconds) {
  using namespace zg;
  if (!s) return 0;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->live.find(ticket);
  if (it == s->live.end()) {
    fail("zfp_gb300_server_wait: unknown ticket");
    return 0;
  }
  std::shared_ptr<Request> r = it->second;
  s->cv.wait(lk, [&] { return r->done; });
  s->live.erase(ticket);
  if (seconds) *seconds = std::chrono::duration<double>(r->t_done - r->t_submit).count();
  if (!r->size) fail("zfp_gb300_server_wait: request failed");
  return r->size;
}

int zfp_gb300_server_stats(zfp_gb300_server* s, size_t* peak_bytes, uint64_t* batches, uint64_t* served) {
  if (!s) return 0;
  std::lock_guard<std::mutex> lk(s->mu);
  if (peak_bytes) *peak_bytes = s->peak;
  if (batches) *batches = s->batches;
  if (served) *served = s->served;
  return 1;
}

void zfp_gb300_server_free(zfp_gb300_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  for (auto& l : s->lanes) {
    cudaStreamSynchronize(l->st);
    if (l->host_jobs) cudaFreeHost(l->host_jobs);
    if (l->host_results) cudaFreeHost(l->host_results);
    for (void* p : l->retired) cudaFreeHost(p);
    cudaStreamDestroy(l->st);
  }
  delete s;
}

}  // extern "C"
