// batch.cu -- many fields, one persistent launch per (type, dimensionality).
//
// The reference compresses one field per zfp_compress call; its CUDA backend
// launches one grid per call (src/cuda_zfp/cuZFP.cu:357-414).  For thousands
// of small uneven fields that launch-and-synchronise pattern leaves the GPU
// idle.  A batch instead describes every field as a Job, numbers the tiles of
// all jobs of one (type, dims) group consecutively and runs the group as one
// persistent grid: CTAs take tiles from a counter in order, which keeps the
// look-back of variable-rate jobs deadlock-free and spreads uneven work over
// all SMs.  The launches are captured once in a CUDA graph and replayed.
// The first run autotunes the persistent grid's CTAs per SM and how much of
// each CTA's shared memory stages tile images / stream words (all of the
// room its occupancy leaves, or half of it, which lets more CTAs share an
// SM while more tiles go through global memory): every candidate is timed
// three times and the one with the best median kept.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <tuple>
#include <utility>
#include <vector>

#include "../../include/zfp_gb300.h"
#include "gpu_internal.h"
#include "runtime.h"

namespace zg {

struct BatchGroup {
  int type = 0, dims = 0;
  std::vector<size_t> members;
  uint32_t total_tiles = 0;
  uint32_t tile_words = 0;     // largest tile image of any member
  uint32_t img_words = 0;      // shared-memory part at full staging (see plan_launch in gpu_codec.cu)
  bool lossy = true;           // no member is reversible: the lossy-only multi-job kernels
  bool needs_ticket = false;
  Job* d_jobs = nullptr;       // device copy of this group's jobs (sorted by tile0)
  LaunchScratch sc{};
  void* scratch = nullptr;     // zeroed before every launch
  size_t scratch_bytes = 0;
};

}  // namespace zg

struct zfp_gb300_batch {
  int direction = 0;
  std::vector<zfp_stream*> streams;
  std::vector<zfp_field> fields;       // copies of the caller's descriptors
  std::vector<zg::FieldInfo> info;
  std::vector<zg::Job> jobs;
  std::vector<uint64_t> nominal_end;   // fixed rate: end bit known up front
  std::vector<zg::BatchGroup> groups;
  zg::JobResult* d_results = nullptr;
  uint64_t* d_offsets = nullptr;       // compress: concatenated per-block indexes of variable-rate jobs
  std::vector<size_t> offset_base;     // per job: first entry in d_offsets (or SIZE_MAX)
  std::vector<zg::IndexRef> held;      // decompress: indexes this batch reads (kept until it is freed)
  cudaStream_t own_stream = nullptr;
  cudaStream_t last_stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  cudaStream_t graph_stream = nullptr;
  int ctas_per_sm = 0;
  int stage_pct = 100;                 // share of the staging room used (100 or 50)
  bool tuned = false;
};

namespace zg {

static int sm_count() { return persistent_grid() / 4; }

static cudaError_t enqueue(zfp_gb300_batch* b, cudaStream_t st, int ctas_per_sm, int stage_pct) {
  for (auto& g : b->groups) {
    cudaError_t e = cudaMemsetAsync(g.scratch, 0, g.scratch_bytes, st);
    if (e != cudaSuccess) return e;
    LaunchArgs a;
    std::memset(&a, 0, sizeof a);
    a.one = b->jobs[g.members[0]];
    a.jobs = g.d_jobs;
    a.njobs = (int)g.members.size();
    a.multi_lossy = g.lossy;
    a.sc = g.sc;
    a.total_tiles = g.total_tiles;
    a.use_ticket = 1;
    // tiles the staging no longer holds are read from the stream (decode)
    // or coded straight into it (encode)
    a.img_words = g.img_words;
    if (stage_pct < 100)
      a.img_words = std::max<uint32_t>(std::min<uint32_t>(64, g.img_words),
                                       (uint32_t)((uint64_t)g.img_words * stage_pct / 100));
    const int grid = std::max(1, sm_count() * ctas_per_sm);
    a.grid = (int)std::min<uint64_t>(g.total_tiles, (uint64_t)grid);
    e = b->direction == 0 ? launch_encode_any(g.type, g.dims, a, st) : launch_decode_any(g.type, g.dims, a, st);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

static void destroy(zfp_gb300_batch* b) {
  if (!b) return;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->last_stream) cudaStreamSynchronize(b->last_stream);
  for (auto& g : b->groups) {
    cudaFree(g.d_jobs);
    cudaFree(g.scratch);
  }
  cudaFree(b->d_results);
  cudaFree(b->d_offsets);
  b->held.clear();
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  delete b;
}

}  // namespace zg

extern "C" {

zfp_gb300_batch* zfp_gb300_batch_create(zfp_stream* const* streams, const zfp_field* const* fields, size_t count,
                                        int direction) {
  using namespace zg;
  if (!count || !streams || !fields || (direction != 0 && direction != 1)) {
    fail("zfp_gb300_batch_create: bad arguments");
    return nullptr;
  }
  init_pool_once();
  zfp_gb300_batch* b = new zfp_gb300_batch();
  b->direction = direction;
  b->streams.assign(streams, streams + count);
  b->fields.resize(count);
  b->info.resize(count);
  b->jobs.resize(count);
  b->nominal_end.assign(count, 0);
  b->offset_base.assign(count, SIZE_MAX);
  cudaError_t e = cudaMalloc((void**)&b->d_results, count * sizeof(JobResult));
  if (e != cudaSuccess) {
    fail_cuda("zfp_gb300_batch_create", e);
    destroy(b);
    return nullptr;
  }
  size_t offset_words = 0;
  std::map<std::tuple<int, int, bool>, size_t> group_of;   // (type, dims, reversible)
  for (size_t i = 0; i < count; i++) {
    zfp_stream* z = streams[i];
    const zfp_field* f = fields[i];
    b->fields[i] = *f;
    FieldInfo& fi = b->info[i];
    const char* why = field_info(f, fi);
    if (why || !z || !z->stream || !is_device_ptr(f->data)) {
      fail(why ? why : "zfp_gb300_batch_create: fields and streams must be in device memory");
      destroy(b);
      return nullptr;
    }
    const StreamState ss = get_stream_state(z->stream);
    if (!ss.begin || !is_device_ptr(ss.begin)) {
      fail("zfp_gb300_batch_create: fields and streams must be in device memory");
      destroy(b);
      return nullptr;
    }
    const bool fixed = is_fixed_rate(fi, z);
    Job j = base_job(fi, z, f->data);
    j.flags = (fixed ? kFixedRate : 0u) | vector_flags(fi, f->data);
    j.words = ss.begin;
    j.cap_words = (uint64_t)(ss.end - ss.begin);
    j.result = b->d_results + i;
    if (direction == 0) {
      j.bit0 = (uint64_t)(ss.ptr - ss.begin) * 64 + ss.bits;
      j.head_word = ss.bits ? (ss.buffer & ((1ull << ss.bits) - 1)) : 0;
      if (fixed) {
        b->nominal_end[i] = j.bit0 + fi.nblocks * (uint64_t)z->maxbits;
        if ((b->nominal_end[i] + 63) / 64 > j.cap_words) {
          fail("zfp_gb300_batch_create: a stream buffer is too small");
          destroy(b);
          return nullptr;
        }
      } else {
        b->offset_base[i] = offset_words;
        offset_words += fi.nblocks;
        j.flags |= kWriteIndex;
      }
    } else {
      j.bit0 = (uint64_t)(ss.ptr - ss.begin) * 64 - ss.bits;
      if (fixed) {
        b->nominal_end[i] = j.bit0 + fi.nblocks * (uint64_t)z->maxbits;
      } else {
        IndexEntry ent;
        if (registry_find(ss.begin, j.bit0, fi, z, ent)) {
          j.offsets = ent.index->ptr;
          j.end_bit = ent.end_bit;
          j.flags |= kVerify;
          b->held.push_back(ent.index);
        } else {
          // stream written elsewhere: recover its block offsets now
          JobResult r{};
          IndexRef idx = make_index(fi.nblocks, nullptr, e);
          if (!idx) {
            fail_cuda("zfp_gb300_batch_create: index", e);
            destroy(b);
            return nullptr;
          }
          Job pj = j;
          pj.offsets = idx->ptr;
          if ((e = cudaMemset(j.result, 0, sizeof(JobResult))) != cudaSuccess ||
              (e = launch_parse_any(fi.type, fi.dims, pj, nullptr)) != cudaSuccess ||
              (e = cudaMemcpy(&r, j.result, sizeof r, cudaMemcpyDeviceToHost)) != cudaSuccess) {
            fail_cuda("zfp_gb300_batch_create: parse", e);
            destroy(b);
            return nullptr;
          }
          j.offsets = idx->ptr;
          j.end_bit = r.end_bit;
          b->held.push_back(idx);
          registry_insert(make_entry(ss.begin, j.bit0, r.end_bit, fi, j, idx));
        }
      }
    }
    b->jobs[i] = j;
    const bool rev = z->minexp < ZFP_MIN_EXP;
    const auto key = std::make_tuple(fi.type, fi.dims, rev);
    auto it = group_of.find(key);
    if (it == group_of.end()) {
      it = group_of.emplace(key, b->groups.size()).first;
      b->groups.emplace_back();
      b->groups.back().type = fi.type;
      b->groups.back().dims = fi.dims;
      b->groups.back().lossy = !rev;
    }
    BatchGroup& g = b->groups[it->second];
    b->jobs[i].tile0 = g.total_tiles;
    g.total_tiles += b->jobs[i].ntiles;
    const uint64_t bound = fixed ? (uint64_t)z->maxbits : block_bound(fi, z);
    g.tile_words = std::max<uint32_t>(g.tile_words, (uint32_t)image_words((uint64_t)kTile * bound / 64 + 4));
    g.members.push_back(i);
  }
  if (offset_words) {
    if ((e = cudaMalloc((void**)&b->d_offsets, offset_words * 8)) != cudaSuccess) {
      fail_cuda("zfp_gb300_batch_create: index", e);
      destroy(b);
      return nullptr;
    }
    for (size_t i = 0; i < count; i++)
      if (b->offset_base[i] != SIZE_MAX) b->jobs[i].offsets = b->d_offsets + b->offset_base[i];
  }
  for (auto& g : b->groups) {
    std::vector<Job> gj;
    for (size_t i : g.members) gj.push_back(b->jobs[i]);
    const size_t t = (size_t)g.total_tiles + 1;
    g.scratch_bytes = 64 + t * 8 + t * 16 + t * 4 + 16;
    if ((e = cudaMalloc((void**)&g.d_jobs, gj.size() * sizeof(Job))) != cudaSuccess ||
        (e = cudaMemcpy(g.d_jobs, gj.data(), gj.size() * sizeof(Job), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMalloc(&g.scratch, g.scratch_bytes)) != cudaSuccess) {
      fail_cuda("zfp_gb300_batch_create: setup", e);
      destroy(b);
      return nullptr;
    }
    char* p = (char*)g.scratch;
    g.sc.ticket = (unsigned int*)(p + 32);
    g.sc.tile_state = (unsigned long long*)(p + 64);
    g.sc.side = (unsigned long long*)(p + 64 + t * 8);
    g.sc.side_cnt = (unsigned int*)(p + 64 + t * 24);
    g.sc.wait_cycles = wait_cycles();
    LaunchArgs probe;
    std::memset(&probe, 0, sizeof probe);
    probe.jobs = g.d_jobs;
    probe.multi_lossy = g.lossy;
    const uint32_t room = stage_room_any(g.type, g.dims, probe, b->direction == 0);
    g.img_words = std::min(g.tile_words, room);
  }
  set_error("");
  return b;
}

zfp_bool zfp_gb300_batch_set_ctas_per_sm(zfp_gb300_batch* b, int ctas_per_sm) {
  if (!b || ctas_per_sm < 0 || ctas_per_sm > 16) return zfp_false;
  b->ctas_per_sm = ctas_per_sm;
  b->stage_pct = 100;
  b->tuned = ctas_per_sm > 0;
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  return zfp_true;
}

zfp_bool zfp_gb300_batch_get_tuning(const zfp_gb300_batch* b, int* ctas_per_sm, int* staging_pct) {
  if (!b || !b->tuned) return zfp_false;
  if (ctas_per_sm) *ctas_per_sm = b->ctas_per_sm;
  if (staging_pct) *staging_pct = b->stage_pct;
  return zfp_true;
}

zfp_bool zfp_gb300_batch_run(zfp_gb300_batch* b, void* cuda_stream) {
  using namespace zg;
  if (!b) return zfp_false;
  cudaStream_t st = (cudaStream_t)cuda_stream;
  cudaError_t e;
  if (!st) {  // the legacy stream cannot be captured: use the batch's own stream
    if (!b->own_stream && (e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking)) != cudaSuccess) {
      fail_cuda("zfp_gb300_batch_run", e);
      return zfp_false;
    }
    st = b->own_stream;
  }
  if (!b->tuned) {
    // autotune: CTAs per SM x staging depth, three timed runs each, best median
    const int ctas[] = {1, 2, 3, 4, 6, 8};
    const int stages[] = {100, 50};
    float best = 1e30f;
    int pick_c = 4, pick_s = 100;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    if ((e = enqueue(b, st, 4, 100)) != cudaSuccess) {  // warm-up (also sets kernel attributes before capture)
      fail_cuda("zfp_gb300_batch_run", e);
      return zfp_false;
    }
    for (int sp : stages)
      for (int c : ctas) {
        float t[3];
        for (float& ms : t) {
          cudaEventRecord(e0, st);
          if ((e = enqueue(b, st, c, sp)) != cudaSuccess) {
            fail_cuda("zfp_gb300_batch_run", e);
            return zfp_false;
          }
          cudaEventRecord(e1, st);
          cudaEventSynchronize(e1);
          cudaEventElapsedTime(&ms, e0, e1);
        }
        std::sort(t, t + 3);
        if (t[1] < best) {
          best = t[1];
          pick_c = c;
          pick_s = sp;
        }
      }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->ctas_per_sm = pick_c;
    b->stage_pct = pick_s;
    b->tuned = true;
  }
  if (!b->graph || b->graph_stream != st) {
    if (b->graph) {
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
    cudaGraph_t g;
    if ((e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
      fail_cuda("zfp_gb300_batch_run: capture", e);
      return zfp_false;
    }
    cudaError_t le = enqueue(b, st, b->ctas_per_sm, b->stage_pct);
    e = cudaStreamEndCapture(st, &g);
    if (le != cudaSuccess || e != cudaSuccess) {
      fail_cuda("zfp_gb300_batch_run: capture", le != cudaSuccess ? le : e);
      return zfp_false;
    }
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      b->graph = nullptr;
      fail_cuda("zfp_gb300_batch_run: instantiate", e);
      return zfp_false;
    }
    b->graph_stream = st;
  }
  if ((e = cudaGraphLaunch(b->graph, st)) != cudaSuccess) {
    fail_cuda("zfp_gb300_batch_run: launch", e);
    return zfp_false;
  }
  b->last_stream = st;
  return zfp_true;
}

zfp_bool zfp_gb300_batch_finish(zfp_gb300_batch* b, size_t* sizes) {
  using namespace zg;
  if (!b || !b->last_stream) return zfp_false;
  cudaError_t e = cudaStreamSynchronize(b->last_stream);
  if (e != cudaSuccess) {
    fail_cuda("zfp_gb300_batch_finish", e);
    return zfp_false;
  }
  std::vector<JobResult> res(b->jobs.size());
  if ((e = cudaMemcpy(res.data(), b->d_results, res.size() * sizeof(JobResult), cudaMemcpyDeviceToHost)) !=
      cudaSuccess) {
    fail_cuda("zfp_gb300_batch_finish", e);
    return zfp_false;
  }
  bool all = true;
  for (size_t i = 0; i < b->jobs.size(); i++) {
    const Job& j = b->jobs[i];
    const bool fixed = j.flags & kFixedRate;
    uint64_t end = 0;
    if (res[i].status) {
      all = false;
      if (sizes) sizes[i] = 0;
      continue;
    }
    if (b->direction == 0) {
      end = fixed ? b->nominal_end[i] : res[i].end_bit;
      const StreamState ss = get_stream_state(b->streams[i]->stream);
      if (!fixed) {  // keep the block index for later decompression of this stream
        cudaError_t ie;
        IndexRef idx = make_index(j.nblocks, b->last_stream, ie);
        if (idx && cudaMemcpyAsync(idx->ptr, j.offsets, j.nblocks * 8, cudaMemcpyDeviceToDevice, b->last_stream) ==
                       cudaSuccess &&
            cudaEventCreateWithFlags(&idx->written, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventRecord(idx->written, b->last_stream) == cudaSuccess)
          registry_insert(make_entry(ss.begin, j.bit0, end, b->info[i], j, idx));
        else
          cudaGetLastError();
      } else {
        registry_invalidate(ss.begin, j.bit0, end);
      }
    } else {
      end = fixed ? b->nominal_end[i] : j.end_bit;
    }
    set_stream_flushed(b->streams[i]->stream, end);
    if (sizes) sizes[i] = (size_t)((end + 63) / 64) * 8;
  }
  if (!all) {
    fail("zfp_gb300_batch_finish: at least one field failed (stream buffer too small or stale index)");
    return zfp_false;
  }
  set_error("");
  return zfp_true;
}

void zfp_gb300_batch_free(zfp_gb300_batch* b) { zg::destroy(b); }

}  // extern "C"
