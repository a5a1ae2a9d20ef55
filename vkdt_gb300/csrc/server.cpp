// The develop server: continuous batching of develop jobs on one device (the
// export daemon beside vkdt-cli; the reference runs one graph at a time).
//
// Jobs are queued by submit(). One worker thread admits them while fewer
// than `slots` are in flight and the device bytes of the pooled graphs stay
// under the cap, runs each on a graph of its shape taken from the pool (one
// CUDA stream per graph, so admitted jobs overlap on the device) and retires
// them by polling their completion events. A graph is allocated when no idle
// graph of the job's shape exists; idle graphs of other shapes are freed,
// least recently used first, when a new one would not fit under the cap.
// Each job runs the same kernels on its own buffers as it would alone, so its
// result does not depend on what else is in flight.
//
// The server is a client of the graph C-ABI: it only calls the functions of
// include/vkdt_cuda.h (and the CUDA runtime for copies and events).
#include "vkdt_cuda.h"
#include "internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace {

using clk = std::chrono::steady_clock;

double ms_between(clk::time_point a, clk::time_point b)
{
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct pooled_t
{
  vkdt_cuda_graph_t *g = nullptr;
  std::vector<int64_t> key;     // shape the graph is allocated for
  uint64_t bytes = 0;
  bool busy = false;
  clk::time_point last;
  cudaEvent_t done = nullptr;   // after the job's last copy
  void *d_src = nullptr, *d_dst = nullptr;  // the graph's own source and sink
  size_t src_bytes = 0, dst_bytes = 0;
  float white[4] = { 0, 0, 0, 0 };          // colour:white as configured (commit_params writes it back)
};

struct job_rec_t
{
  vkdt_cuda_job_t job;
  int status = VKDT_CUDA_NOT_READY;
  std::string err;
  bool started = false, done = false;
  int slot = -1;                // index into the pool while running
  clk::time_point t_submit, t_start, t_done;
};

dt_token_t tok(const char *s)
{ // src/pipe/token.h: up to 8 characters packed little endian
  uint64_t t = 0;
  for(int i = 0; i < 8 && s[i]; i++) t |= ((uint64_t)(uint8_t)s[i]) << (8 * i);
  return t;
}

std::vector<int64_t> shape_key(const vkdt_cuda_job_t &j)
{
  return { j.wd, j.ht, (int64_t)j.ip.filters, (int64_t)j.ip.crop_aabb[0], (int64_t)j.ip.crop_aabb[1],
           (int64_t)j.ip.crop_aabb[2], (int64_t)j.ip.crop_aabb[3], j.out_wd, j.out_ht };
}

} // namespace

struct vkdt_cuda_server_t
{
  std::string cfg;
  bool have_cfg = false;
  int slots = 1, llap_levels = 0, device = 0;
  uint64_t cap = 0;
  std::mutex m;
  std::condition_variable cv_work, cv_done;
  std::deque<uint64_t> queue;
  std::map<uint64_t, job_rec_t> jobs;
  std::vector<pooled_t> pool;
  int running = 0;
  std::vector<uint64_t> inflight;   // started, not retired
  uint64_t next_id = 1, bytes = 0, peak = 0, completed = 0, failed = 0;
  double mpix = 0.0;
  std::vector<double> lat;
  bool stop = false;
  std::thread worker;

  // graph for a job's shape: an idle pooled one, or a new one if it fits. -1: wait, -2: cannot ever fit
  int acquire(const job_rec_t &r, std::string &err, int &code)
  {
    code = VKDT_CUDA_ERROR_OUT_OF_DEVICE_MEMORY;
    const std::vector<int64_t> key = shape_key(r.job);
    for(size_t i = 0; i < pool.size(); i++)
      if(!pool[i].busy && pool[i].key == key) return (int)i;
    vkdt_cuda_graph_t *g = nullptr;
    int rc = vkdt_cuda_graph_create(&g);
    if(!rc && have_cfg) rc = vkdt_cuda_graph_read_config(g, cfg.data(), cfg.size());
    if(!rc && llap_levels) rc = vkdt_cuda_graph_set_llap_levels(g, llap_levels);
    if(!rc) rc = vkdt_cuda_graph_set_input(g, r.job.wd, r.job.ht, &r.job.ip);
    if(!rc && (r.job.out_wd || r.job.out_ht)) rc = vkdt_cuda_graph_set_output_size(g, r.job.out_wd, r.job.out_ht);
    float white[4] = { 0, 0, 0, 0 };
    if(!rc) rc = vkdt_cuda_graph_get_param(g, tok("colour"), tok("01"), tok("white"), white, sizeof(white));
    uint64_t need = 0;
    if(!rc) rc = vkdt_cuda_graph_plan_bytes(g, &need);
    if(rc) { err = vkdt_cuda_last_error(); code = rc; vkdt_cuda_graph_destroy(g); return -2; }
    if(need > cap) { err = "job needs more device memory than the server's cap"; vkdt_cuda_graph_destroy(g); return -2; }
    // free idle graphs of other shapes, least recently used first, until it fits
    while(bytes + need > cap)
    {
      int lru = -1;
      for(size_t i = 0; i < pool.size(); i++)
        if(!pool[i].busy && (lru < 0 || pool[i].last < pool[lru].last)) lru = (int)i;
      if(lru < 0) { vkdt_cuda_graph_destroy(g); return -1; }   // everything is busy: wait
      release(lru);
    }
    uint64_t got = 0;
    // every job replays the graph's captured launch sequence, updated in place for its buffers and metadata
    rc = vkdt_cuda_graph_alloc(g, &got);
    pooled_t p;
    if(!rc) rc = vkdt_cuda_graph_device_buffers(g, &p.d_src, &p.d_dst);
    if(!rc && cudaEventCreateWithFlags(&p.done, cudaEventDisableTiming) != cudaSuccess) rc = VKDT_CUDA_ERROR_UNKNOWN;
    if(rc) { err = vkdt_cuda_last_error(); code = rc; vkdt_cuda_graph_destroy(g); return -2; }
    int ow = 0, oh = 0;
    vkdt_cuda_graph_output_size(g, &ow, &oh);
    p.g = g; p.key = key; p.bytes = got; p.last = clk::now();
    memcpy(p.white, white, sizeof(white));
    p.src_bytes = (size_t)r.job.wd * r.job.ht * 2;
    p.dst_bytes = (size_t)ow * oh * 8;
    pool.push_back(p);
    bytes += got;
    peak = std::max(peak, bytes);
    return (int)pool.size() - 1;
  }

  void release(int i)
  {
    pooled_t &p = pool[i];
    if(p.done) cudaEventDestroy(p.done);
    vkdt_cuda_graph_destroy(p.g);
    bytes -= p.bytes;
    pool.erase(pool.begin() + i);
    for(uint64_t id : inflight) if(jobs[id].slot > i) jobs[id].slot--;
  }

  // enqueue the copies and kernels of a job on its graph's stream
  int start(job_rec_t &r, int slot)
  {
    pooled_t &p = pool[slot];
    vkdt_cuda_graph_t *g = p.g;
    int rc = vkdt_cuda_graph_set_input(g, r.job.wd, r.job.ht, &r.job.ip);   // same shape: new metadata only
    // colour/main.c:241-253 derives the white from this image's camera coefficients when the
    // configured white is 0 and writes it back: restore the configured value for every image
    if(!rc) rc = vkdt_cuda_graph_set_param(g, tok("colour"), tok("01"), tok("white"), p.white, sizeof(p.white));
    if(rc) return rc;
    cudaStream_t s = (cudaStream_t)vkdt_cuda_graph_stream(g);
    const void *src = r.job.src;
    if(!r.job.src_on_device)
    {
      if(cudaMemcpyAsync(p.d_src, r.job.src, p.src_bytes, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return vkdt_set_error(VKDT_CUDA_ERROR_DEVICE_LOST, "upload failed");
      src = p.d_src;
    }
    void *dst = r.job.dst_on_device ? r.job.dst : p.d_dst;
    rc = vkdt_cuda_graph_develop(g, src, dst, s);
    if(rc) return rc;
    if(!r.job.dst_on_device && cudaMemcpyAsync(r.job.dst, p.d_dst, p.dst_bytes, cudaMemcpyDeviceToHost, s) != cudaSuccess)
      return vkdt_set_error(VKDT_CUDA_ERROR_DEVICE_LOST, "download failed");
    if(cudaEventRecord(p.done, s) != cudaSuccess) return vkdt_set_error(VKDT_CUDA_ERROR_DEVICE_LOST, "event record failed");
    return 0;
  }

  void finish(job_rec_t &r, int status, const std::string &err)
  {
    r.status = status;
    r.err = err;
    r.done = true;
    r.t_done = clk::now();
    if(r.slot >= 0) { pool[r.slot].busy = false; pool[r.slot].last = r.t_done; }
    r.slot = -1;
    running--;
    if(status == 0)
    {
      completed++;
      mpix += (double)r.job.wd * r.job.ht * 1e-6;
      lat.push_back(ms_between(r.t_submit, r.t_done));
    }
    else failed++;
  }

  void run()
  {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(m);
    while(true)
    {
      // retire finished jobs
      for(size_t k = 0; k < inflight.size();)
      {
        job_rec_t &r = jobs[inflight[k]];
        const cudaError_t e = cudaEventQuery(pool[r.slot].done);
        if(e == cudaErrorNotReady) { k++; continue; }
        finish(r, e == cudaSuccess ? 0 : VKDT_CUDA_ERROR_DEVICE_LOST, e == cudaSuccess ? "" : cudaGetErrorString(e));
        inflight.erase(inflight.begin() + k);
        cv_done.notify_all();
      }
      // admit queued jobs
      while(running < slots && !queue.empty())
      {
        const uint64_t r_id = queue.front();
        job_rec_t &r = jobs[r_id];
        std::string err;
        int code = 0;
        const int slot = acquire(r, err, code);
        if(slot == -1) break;                   // wait for a graph to become idle
        queue.pop_front();
        r.started = true;
        r.t_start = clk::now();
        running++;
        if(slot < 0) { finish(r, code, err); cv_done.notify_all(); continue; }
        r.slot = slot;
        pool[slot].busy = true;
        const int rc = start(r, slot);
        if(rc) { finish(r, rc, vkdt_cuda_last_error()); cv_done.notify_all(); }
        else inflight.push_back(r_id);
      }
      if(stop && queue.empty() && running == 0) break;
      // poll the device while jobs run, sleep until a submit otherwise
      if(running > 0) cv_work.wait_for(lk, std::chrono::microseconds(50));
      else cv_work.wait(lk, [&] { return stop || !queue.empty(); });
    }
  }
};

#pragma GCC visibility push(default)
extern "C" {

int vkdt_cuda_server_create(const vkdt_cuda_server_cfg_t *cfg, vkdt_cuda_server_t **server)
{
  if(!cfg || !server || cfg->slots < 1) return vkdt_set_error(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "bad server config");
  int dev = 0;
  if(cudaGetDevice(&dev) != cudaSuccess) return vkdt_set_error(VKDT_CUDA_ERROR_INITIALIZATION_FAILED, "no CUDA device");
  vkdt_cuda_server_t *s = new vkdt_cuda_server_t;
  if(cfg->cfg) { s->cfg.assign(cfg->cfg, cfg->cfg_len); s->have_cfg = true; }
  s->slots = cfg->slots;
  s->llap_levels = cfg->llap_levels;
  s->device = dev;
  s->cap = cfg->hbm_cap;
  if(!s->cap)
  {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    s->cap = (uint64_t)(0.9 * fr);
  }
  s->worker = std::thread([s] { s->run(); });
  *server = s;
  return 0;
}

int vkdt_cuda_server_submit(vkdt_cuda_server_t *s, const vkdt_cuda_job_t *job, uint64_t *job_id)
{
  if(!s || !job || !job->src || !job->dst || job->wd <= 0 || job->ht <= 0)
    return vkdt_set_error(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "bad job");
  std::lock_guard<std::mutex> lk(s->m);
  const uint64_t id = s->next_id++;
  job_rec_t &r = s->jobs[id];
  r.job = *job;
  r.t_submit = clk::now();
  s->queue.push_back(id);
  if(job_id) *job_id = id;
  s->cv_work.notify_one();
  return 0;
}

int vkdt_cuda_server_wait(vkdt_cuda_server_t *s, uint64_t id, uint32_t timeout_ms)
{
  if(!s) return vkdt_set_error(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "null server");
  std::unique_lock<std::mutex> lk(s->m);
  auto it = s->jobs.find(id);
  if(it == s->jobs.end()) return vkdt_set_error(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "no such job");
  if(!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return it->second.done; }))
    return timeout_ms ? vkdt_set_error(VKDT_CUDA_TIMEOUT, "job not done in time") : VKDT_CUDA_NOT_READY;
  if(it->second.status) return vkdt_set_error(it->second.status, it->second.err.c_str());
  return 0;
}

int vkdt_cuda_server_drain(vkdt_cuda_server_t *s, uint32_t timeout_ms)
{
  if(!s) return vkdt_set_error(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "null server");
  std::unique_lock<std::mutex> lk(s->m);
  if(!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return s->queue.empty() && s->running == 0; }))
    return vkdt_set_error(VKDT_CUDA_TIMEOUT, "jobs still running");
  return 0;
}

int vkdt_cuda_server_job_times(vkdt_cuda_server_t *s, uint64_t id, double *queued_ms, double *latency_ms)
{
  if(!s) return vkdt_set_error(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "null server");
  std::lock_guard<std::mutex> lk(s->m);
  auto it = s->jobs.find(id);
  if(it == s->jobs.end()) return vkdt_set_error(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "no such job");
  if(!it->second.done) return VKDT_CUDA_NOT_READY;
  if(queued_ms) *queued_ms = ms_between(it->second.t_submit, it->second.t_start);
  if(latency_ms) *latency_ms = ms_between(it->second.t_submit, it->second.t_done);
  return 0;
}

int vkdt_cuda_server_stats(vkdt_cuda_server_t *s, vkdt_cuda_server_stats_t *st)
{
  if(!s || !st) return vkdt_set_error(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "null argument");
  std::lock_guard<std::mutex> lk(s->m);
  memset(st, 0, sizeof(*st));
  st->completed = s->completed;
  st->failed = s->failed;
  st->mpix = s->mpix;
  st->peak_device_bytes = s->peak;
  st->graphs = (int)s->pool.size();
  if(!s->lat.empty())
  {
    std::vector<double> l = s->lat;
    std::sort(l.begin(), l.end());
    auto pct = [&](double q) { // nearest rank
      size_t k = (size_t)std::ceil(q * l.size());
      return l[std::min(l.size() - 1, k ? k - 1 : 0)];
    };
    st->latency_p50_ms = pct(0.50);
    st->latency_p99_ms = pct(0.99);
  }
  return 0;
}

int vkdt_cuda_server_reset_stats(vkdt_cuda_server_t *s)
{
  if(!s) return vkdt_set_error(VKDT_CUDA_ERROR_FORMAT_NOT_SUPPORTED, "null server");
  std::lock_guard<std::mutex> lk(s->m);
  s->completed = s->failed = 0;
  s->mpix = 0.0;
  s->lat.clear();
  s->peak = s->bytes;
  for(auto it = s->jobs.begin(); it != s->jobs.end();) it = it->second.done ? s->jobs.erase(it) : std::next(it);
  return 0;
}

void vkdt_cuda_server_destroy(vkdt_cuda_server_t *s)
{
  if(!s) return;
  {
    std::lock_guard<std::mutex> lk(s->m);
    s->stop = true;
    s->cv_work.notify_all();
  }
  s->worker.join();
  while(!s->pool.empty()) s->release((int)s->pool.size() - 1);
  delete s;
}

} // extern "C"
#pragma GCC visibility pop
