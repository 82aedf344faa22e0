// Serving loop for CC iteration requests (include/gbx_serve.h).
//
// Host threads: the dispatcher (the caller of gbx_server_run) polls
// completion events, admits waiting jobs by planned footprint against the
// byte budget, and puts the earliest runnable request on every free stream
// slot: one graph launch of the job's iteration, an asynchronous read of its
// energy into pinned memory, then an event.  Three builder threads create
// admitted jobs (host planning, integrals, constant operands, graph capture;
// up to three at once, so one large job does not hold up the others), evict
// idle jobs and check and destroy finished ones, so that none of this stalls
// dispatch.
//
// Idle jobs do not hold the budget: when a job waiting for admission does
// not fit, resident jobs with no request waiting (least recently used first)
// are evicted -- their amplitudes saved to pinned host memory, their device
// state released -- and an evicted job is admitted again, rebuilt and given
// its saved amplitudes back, when its next request arrives.  The iterations
// after a restore repeat those of a job that never left the device.
//
// Job state comes from the stream-ordered allocator on a stream of the
// server's own, so releasing a finished job does not wait for the whole
// device (cudaFree would, and with other jobs' iterations always in flight
// that wait has no end in sight).  Job creation runs on the legacy default
// stream; the slots are non-blocking streams, so the two never wait on each
// other implicitly.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/gbx_serve.h"
#include "common.h"

namespace {

using Clock = std::chrono::steady_clock;

constexpr int kPending = 1;  // request status while it has not finished
constexpr int kBuilders = 3;  // builder threads: job builds in flight at once

struct Req {
  int job = 0, iter = 0;
  double arrival = 0.0, start = 0.0, end = 0.0, energy = 0.0;
  int status = kPending, slot = -1;
};

enum class JobState { Waiting, Building, Ready, Busy, Finished, Rejected, Evicting, Evicted };

struct Job {
  gbx_cc_config cfg;
  double footprint = 0.0, measured = 0.0;
  std::vector<int> reqs;  // request indices in iteration (arrival) order
  int next = 0, done = 0;
  JobState state = JobState::Waiting;
  gbx_cc_job* h = nullptr;
  int build_status = GBX_OK, check_status = GBX_OK;
  double build_s = 0.0;
  double last_done = 0.0;  // when its last request finished (eviction order)
  // amplitudes saved in pinned host memory while the job is evicted
  double* h_t1 = nullptr;
  double* h_t2 = nullptr;
  int64_t n1 = 0, n2 = 0;
  bool saved = false;
  double evict_s = 0.0;
  int evict_status = GBX_OK;
  void free_saved() {
    if (h_t1) cudaFreeHost(h_t1);
    if (h_t2) cudaFreeHost(h_t2);
    h_t1 = h_t2 = nullptr;
    saved = false;
  }
};

double pct(std::vector<double> v, double q) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double pos = q * (double)(v.size() - 1);
  const size_t i = (size_t)pos;
  const double f = pos - (double)i;
  return i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

}  // namespace

struct gbx_server {
  gbx_serve_config cfg;
  std::vector<Job> jobs;
  std::vector<Req> reqs;
  gbx_serve_stats stats;
  bool ran = false;
  int device = 0;
  cudaStream_t mem_stream = nullptr;  // stream-ordered allocations of job state
  // builder threads' queues (guarded by mu)
  std::mutex mu;
  std::condition_variable cv;
  std::deque<int> to_build, to_destroy, to_evict;
  std::vector<int> built, destroyed, evicted;
  bool stop = false;

  // Saves an idle job's amplitudes to pinned host memory and releases its
  // device state (a builder thread).
  int evict(Job& j) {
    int rc = gbx_cc_amplitude_elems(j.h, &j.n1, &j.n2);
    if (rc == GBX_OK && !j.h_t2) {
      if (cudaMallocHost((void**)&j.h_t2, sizeof(double) * std::max<int64_t>(j.n2, 1)) != cudaSuccess ||
          cudaMallocHost((void**)&j.h_t1, sizeof(double) * std::max<int64_t>(j.n1, 1)) != cudaSuccess)
        rc = gbx::fail(GBX_ENOMEM, "pinned host memory for evicted amplitudes");
    }
    if (rc == GBX_OK) rc = gbx_cc_save_amplitudes(j.h, j.n1 ? j.h_t1 : nullptr, j.h_t2, nullptr);
    if (rc == GBX_OK && cudaStreamSynchronize(nullptr) != cudaSuccess)
      rc = gbx::fail(GBX_ECUDA, "saving amplitudes failed");
    const int chk = gbx_cc_check(j.h);
    if (rc == GBX_OK) rc = chk;
    gbx_cc_destroy(j.h);
    j.saved = rc == GBX_OK;
    return rc;
  }

  void builder() {
    cudaSetDevice(device);
    gbx::StreamOrderedAlloc ordered(mem_stream);
    for (;;) {
      int b = -1, d = -1;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return stop || !to_build.empty() || !to_destroy.empty() || !to_evict.empty(); });
        if (!to_destroy.empty()) {
          d = to_destroy.front();
          to_destroy.pop_front();
        } else if (!to_evict.empty()) {
          const int e = to_evict.front();
          to_evict.pop_front();
          lk.unlock();
          Job& j = jobs[e];
          const auto t0 = Clock::now();
          const int rc = evict(j);
          lk.lock();
          j.h = nullptr;
          j.evict_status = rc;
          j.evict_s = std::chrono::duration<double>(Clock::now() - t0).count();
          evicted.push_back(e);
          continue;
        } else if (!to_build.empty()) {
          b = to_build.front();
          to_build.pop_front();
        } else {
          return;  // stop requested and nothing left
        }
      }
      if (d >= 0) {
        Job& j = jobs[d];
        // every request of the job has completed: read the error words of
        // its bounded device waits, then release the state
        const int st = gbx_cc_check(j.h);
        gbx_cc_destroy(j.h);
        j.free_saved();
        std::lock_guard<std::mutex> lk(mu);
        j.h = nullptr;
        j.check_status = st;
        destroyed.push_back(d);
      }
      if (b >= 0) {
        Job& j = jobs[b];
        const auto t0 = Clock::now();
        gbx_cc_job* h = nullptr;
        int rc = gbx_cc_create(&j.cfg, nullptr, &h);
        if (rc == GBX_OK) rc = gbx_cc_capture(h);
        if (rc == GBX_OK && j.saved) {
          // an evicted job comes back with the amplitudes it left with
          rc = gbx_cc_set_amplitudes(h, j.n1 ? j.h_t1 : nullptr, j.h_t2, nullptr);
          if (rc == GBX_OK && cudaStreamSynchronize(nullptr) != cudaSuccess)
            rc = gbx::fail(GBX_ECUDA, "restoring amplitudes failed");
        }
        double meas = 0.0;
        if (rc == GBX_OK) {
          gbx_cc_stats st;
          if (gbx_cc_stats_get(h, &st) == GBX_OK) meas = st.resident_bytes;
        } else if (h) {
          gbx_cc_destroy(h);
          h = nullptr;
        }
        const double dt = std::chrono::duration<double>(Clock::now() - t0).count();
        std::lock_guard<std::mutex> lk(mu);
        j.h = h;
        j.measured = meas;
        j.build_s = dt;
        j.build_status = rc;
        built.push_back(b);
      }
    }
  }
};

using namespace gbx;

extern "C" {

int gbx_server_create(const gbx_serve_config* cfg, gbx_server** out) {
  if (!cfg || !out) return fail(GBX_EINVAL, "null argument");
  *out = nullptr;
  if (!(cfg->budget_bytes > 0) || cfg->slots < 1 || cfg->slots > 64)
    return fail(GBX_EINVAL, "bad serving configuration");
  auto s = new gbx_server();
  s->cfg = *cfg;
  std::memset(&s->stats, 0, sizeof(s->stats));
  *out = s;
  return GBX_OK;
}

int gbx_server_add_job(gbx_server* s, const gbx_cc_config* cfg, int* job_id, double* footprint_bytes) {
  if (!s || !cfg || !job_id) return fail(GBX_EINVAL, "null argument");
  if (s->ran) return fail(GBX_EINVAL, "the server has already run");
  Job j;
  j.cfg = *cfg;
  j.cfg.use_graph = 1;
  GBX_TRY(gbx_cc_footprint(&j.cfg, &j.footprint, nullptr, nullptr));
  s->jobs.push_back(j);
  *job_id = (int)s->jobs.size() - 1;
  if (footprint_bytes) *footprint_bytes = j.footprint;
  return GBX_OK;
}

int gbx_server_submit(gbx_server* s, int job_id, double arrival_s) {
  if (!s || job_id < 0 || job_id >= (int)s->jobs.size() || !(arrival_s >= 0))
    return fail(GBX_EINVAL, "bad request");
  if (s->ran) return fail(GBX_EINVAL, "the server has already run");
  Req r;
  r.job = job_id;
  r.arrival = arrival_s;
  s->reqs.push_back(r);
  return GBX_OK;
}

int gbx_server_run(gbx_server* s, double time_limit_s) {
  if (!s) return fail(GBX_EINVAL, "null server");
  if (s->ran) return fail(GBX_EINVAL, "the server has already run");
  s->ran = true;
  GBX_CUDA(cudaGetDevice(&s->device));
  GBX_CUDA(cudaStreamCreateWithFlags(&s->mem_stream, cudaStreamNonBlocking));
  // a job's requests run in arrival order
  for (size_t i = 0; i < s->reqs.size(); ++i) s->jobs[s->reqs[i].job].reqs.push_back((int)i);
  for (auto& j : s->jobs) {
    std::stable_sort(j.reqs.begin(), j.reqs.end(),
                     [&](int a, int b) { return s->reqs[a].arrival < s->reqs[b].arrival; });
    for (size_t k = 0; k < j.reqs.size(); ++k) s->reqs[j.reqs[k]].iter = (int)k + 1;
  }
  std::vector<int> order(s->reqs.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return s->reqs[a].arrival < s->reqs[b].arrival; });
  std::vector<int> job_order;  // by first arrival
  std::vector<char> seen(s->jobs.size(), 0);
  for (int r : order)
    if (!seen[s->reqs[r].job]) {
      seen[s->reqs[r].job] = 1;
      job_order.push_back(s->reqs[r].job);
    }

  const int nslot = s->cfg.slots;
  std::vector<cudaStream_t> streams(nslot, nullptr);
  std::vector<cudaEvent_t> events(nslot, nullptr);
  std::vector<int> slot_req(nslot, -1);
  double* pinned = nullptr;
  int rc = GBX_OK;
  for (int i = 0; i < nslot && rc == GBX_OK; ++i) {
    if (cudaStreamCreateWithFlags(&streams[i], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&events[i], cudaEventDisableTiming) != cudaSuccess)
      rc = fail(GBX_ECUDA, "stream or event creation failed");
  }
  if (rc == GBX_OK && cudaMallocHost((void**)&pinned, sizeof(double) * nslot) != cudaSuccess)
    rc = fail(GBX_ECUDA, "pinned buffer allocation failed");
  std::vector<std::thread> workers;
  if (rc == GBX_OK)
    for (int b = 0; b < kBuilders; ++b) workers.emplace_back([s] { s->builder(); });

  double planned = 0.0, measured = 0.0;
  int building = 0, evicting = 0, finished_reqs = 0;
  const int total = (int)s->reqs.size();
  const auto t0 = Clock::now();
  auto now = [&] { return std::chrono::duration<double>(Clock::now() - t0).count(); };
  auto finish_job_requests = [&](Job& j, int status) {
    for (int k = j.next; k < (int)j.reqs.size(); ++k) {
      Req& r = s->reqs[j.reqs[k]];
      if (r.status == kPending) {
        r.status = status;
        ++finished_reqs;
      }
    }
    j.next = (int)j.reqs.size();
  };
  // results of the builder threads: builds done, jobs evicted or destroyed
  auto collect = [&]() -> bool {
    bool any = false;
    std::lock_guard<std::mutex> lk(s->mu);
    for (int b : s->built) {
      Job& j = s->jobs[b];
      --building;
      s->stats.build_s_total += j.build_s;
      if (j.build_status == GBX_OK) {
        j.state = JobState::Ready;
        measured += j.measured;
        s->stats.peak_measured_bytes = std::max(s->stats.peak_measured_bytes, measured);
        ++s->stats.jobs_admitted;
      } else {
        j.state = JobState::Rejected;
        planned -= j.footprint;
        finish_job_requests(j, j.build_status);
        ++s->stats.jobs_rejected;
      }
      any = true;
    }
    s->built.clear();
    for (int e : s->evicted) {
      Job& j = s->jobs[e];
      --evicting;
      planned -= j.footprint;
      measured -= j.measured;
      s->stats.evict_s_total += j.evict_s;
      if (j.evict_status == GBX_OK) {
        j.state = JobState::Evicted;
        ++s->stats.evictions;
      } else {
        j.state = JobState::Rejected;
        finish_job_requests(j, j.evict_status);
      }
      any = true;
    }
    s->evicted.clear();
    for (int d : s->destroyed) {
      Job& j = s->jobs[d];
      planned -= j.footprint;
      measured -= j.measured;
      if (j.check_status != GBX_OK)
        for (int k : j.reqs) s->reqs[k].status = j.check_status;
      any = true;
    }
    s->destroyed.clear();
    return any;
  };
  bool timed_out = false;
  while (rc == GBX_OK && finished_reqs < total) {
    const double t = now();
    bool progress = false;
    // completions
    for (int i = 0; i < nslot; ++i) {
      if (slot_req[i] < 0) continue;
      const cudaError_t q = cudaEventQuery(events[i]);
      if (q == cudaErrorNotReady) continue;
      Req& r = s->reqs[slot_req[i]];
      Job& j = s->jobs[r.job];
      r.end = t;
      r.energy = pinned[i];
      r.status = q == cudaSuccess ? GBX_OK : GBX_ECUDA;
      ++finished_reqs;
      ++j.done;
      slot_req[i] = -1;
      progress = true;
      if (q != cudaSuccess) {
        rc = cuda_fail(q, "iteration request", __FILE__, __LINE__);
        break;
      }
      j.last_done = t;
      if (j.done == (int)j.reqs.size()) {
        j.state = JobState::Finished;
        std::lock_guard<std::mutex> lk(s->mu);
        s->to_destroy.push_back(r.job);
        s->cv.notify_one();
      } else {
        j.state = JobState::Ready;
      }
    }
    if (collect()) progress = true;
    // admission: first fit in order of first arrival, up to kBuilders builds at a time;
    // the first job that does not fit may evict idle jobs to make room
    if (building < kBuilders && evicting == 0) {
      bool tried_evict = false;
      for (int jb : job_order) {
        Job& j = s->jobs[jb];
        const bool fresh = j.state == JobState::Waiting && !j.reqs.empty() && s->reqs[j.reqs[0]].arrival <= t;
        const bool back = j.state == JobState::Evicted && j.next < (int)j.reqs.size() &&
                          s->reqs[j.reqs[j.next]].arrival <= t;
        if (!fresh && !back) continue;
        if (j.footprint > s->cfg.budget_bytes) {
          j.state = JobState::Rejected;
          finish_job_requests(j, GBX_ENOMEM);
          ++s->stats.jobs_rejected;
          progress = true;
          continue;
        }
        if (planned + j.footprint > s->cfg.budget_bytes) {
          if (tried_evict) continue;
          tried_evict = true;
          // idle resident jobs: no request of theirs waiting; least recently used first
          std::vector<int> idle;
          for (size_t k = 0; k < s->jobs.size(); ++k) {
            const Job& q = s->jobs[k];
            if (q.state == JobState::Ready && q.next < (int)q.reqs.size() && s->reqs[q.reqs[q.next]].arrival > t)
              idle.push_back((int)k);
          }
          std::sort(idle.begin(), idle.end(),
                    [&](int a, int b) { return s->jobs[a].last_done < s->jobs[b].last_done; });
          double room = s->cfg.budget_bytes - planned;
          std::vector<int> victims;
          for (int k : idle) {
            if (room >= j.footprint) break;
            victims.push_back(k);
            room += s->jobs[k].footprint;
          }
          if (room >= j.footprint && !victims.empty()) {
            std::lock_guard<std::mutex> lk(s->mu);
            for (int k : victims) {
              s->jobs[k].state = JobState::Evicting;
              ++evicting;
              s->to_evict.push_back(k);
            }
            s->cv.notify_one();
            progress = true;
            break;
          }
          continue;
        }
        if (back) ++s->stats.restores;
        planned += j.footprint;
        s->stats.peak_planned_bytes = std::max(s->stats.peak_planned_bytes, planned);
        j.state = JobState::Building;
        ++building;
        std::lock_guard<std::mutex> lk(s->mu);
        s->to_build.push_back(jb);
        s->cv.notify_one();
        progress = true;
        break;
      }
    }
    // dispatch: the earliest arrived runnable request on every free slot
    for (int i = 0; i < nslot && rc == GBX_OK; ++i) {
      if (slot_req[i] >= 0) continue;
      int pick = -1;
      for (int r : order) {
        const Req& q = s->reqs[r];
        if (q.arrival > t) break;
        if (q.status != kPending || q.slot >= 0) continue;
        const Job& j = s->jobs[q.job];
        if (j.state != JobState::Ready || j.reqs[j.next] != r) continue;
        pick = r;
        break;
      }
      if (pick < 0) break;
      Req& q = s->reqs[pick];
      Job& j = s->jobs[q.job];
      rc = gbx_cc_enqueue(j.h, 1, streams[i]);
      if (rc == GBX_OK) rc = gbx_cc_read_energy(j.h, pinned + i, streams[i]);
      if (rc == GBX_OK && cudaEventRecord(events[i], streams[i]) != cudaSuccess)
        rc = fail(GBX_ECUDA, "event record failed");
      if (rc != GBX_OK) break;
      q.start = now();
      q.slot = i;
      ++j.next;
      j.state = JobState::Busy;
      slot_req[i] = pick;
      progress = true;
    }
    if (time_limit_s > 0 && now() > time_limit_s) {
      timed_out = true;
      break;
    }
    if (!progress) std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
  // drain: requests already on the GPU finish; those never started time out
  for (int i = 0; i < nslot; ++i)
    if (streams[i]) cudaStreamSynchronize(streams[i]);
  const double tend = now();
  for (int i = 0; i < nslot; ++i) {
    if (slot_req[i] < 0) continue;
    Req& r = s->reqs[slot_req[i]];
    r.end = tend;
    r.energy = pinned[i];
    r.status = GBX_OK;
    slot_req[i] = -1;
  }
  for (auto& r : s->reqs)
    if (r.status == kPending) r.status = timed_out ? GBX_ETIMEOUT : GBX_EINVAL;
  if (!workers.empty()) {
    // builds still queued or running end first (polled: the builders do not
    // signal this thread), then every job still resident is released
    for (;;) {
      collect();
      if (building <= 0 && evicting <= 0) break;
      std::this_thread::sleep_for(std::chrono::milliseconds(1));
    }
    {
      std::lock_guard<std::mutex> lk(s->mu);
      for (size_t jb = 0; jb < s->jobs.size(); ++jb)
        if (s->jobs[jb].h && s->jobs[jb].state != JobState::Finished) s->to_destroy.push_back((int)jb);
      s->stop = true;
      s->cv.notify_all();
    }
    for (auto& w : workers) w.join();
    collect();
  }
  for (int i = 0; i < nslot; ++i) {
    if (events[i]) cudaEventDestroy(events[i]);
    if (streams[i]) cudaStreamDestroy(streams[i]);
  }
  if (pinned) cudaFreeHost(pinned);
  cudaStreamSynchronize(s->mem_stream);
  // statistics
  gbx_serve_stats& st = s->stats;
  st.requests = total;
  st.jobs = (int)s->jobs.size();
  std::vector<double> lat, svc;
  double first = 1e300, last = 0.0;
  for (auto& r : s->reqs) {
    if (r.status == GBX_OK) {
      ++st.completed;
      lat.push_back(r.end - r.arrival);
      svc.push_back(r.end - r.start);
      first = std::min(first, r.arrival);
      last = std::max(last, r.end);
    } else if (r.status == GBX_ETIMEOUT) {
      ++st.timed_out;
    } else {
      ++st.rejected;
    }
  }
  st.makespan_s = st.completed ? last - first : 0.0;
  st.iter_per_s = st.makespan_s > 0 ? st.completed / st.makespan_s : 0.0;
  st.latency_p50_s = pct(lat, 0.50);
  st.latency_p99_s = pct(lat, 0.99);
  st.latency_max_s = lat.empty() ? 0.0 : *std::max_element(lat.begin(), lat.end());
  st.service_p50_s = pct(svc, 0.50);
  return rc;
}

int gbx_server_results(const gbx_server* s, gbx_serve_result* out, int* count) {
  if (!s || !count) return fail(GBX_EINVAL, "null argument");
  if (!out) {
    *count = (int)s->reqs.size();
    return GBX_OK;
  }
  const int n = std::min(*count, (int)s->reqs.size());
  for (int i = 0; i < n; ++i) {
    const Req& r = s->reqs[i];
    out[i].job = r.job;
    out[i].iteration = r.iter;
    out[i].status = r.status;
    out[i].slot = r.slot;
    out[i].arrival = r.arrival;
    out[i].start = r.start;
    out[i].end = r.end;
    out[i].energy = r.energy;
  }
  *count = n;
  return GBX_OK;
}

int gbx_server_stats(const gbx_server* s, gbx_serve_stats* out) {
  if (!s || !out) return fail(GBX_EINVAL, "null argument");
  *out = s->stats;
  return GBX_OK;
}

int gbx_server_destroy(gbx_server* s) {
  if (s) {
    for (auto& j : s->jobs) {
      if (j.h) gbx_cc_destroy(j.h);
      j.free_saved();
    }
    if (s->mem_stream) {
      cudaStreamSynchronize(s->mem_stream);
      cudaStreamDestroy(s->mem_stream);
    }
    delete s;
  }
  return GBX_OK;
}

}  // extern "C"
