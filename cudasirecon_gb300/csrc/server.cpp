// ReconServer: a FIFO of volume requests served by worker threads, each
// running the plain per-volume flow (setRaw -> loadAndRescaleImage(0) ->
// processOneVolume -> getResult) on a handle it holds for the request, or, for
// a chunk of a batch, the same flow over the chunk's volumes with copies
// overlapped (process_series, standalone form).
//
// Handles are pooled per (configuration, nx, ny, nimages): a worker reuses an
// idle handle of the request's shape, else creates one.  Device memory is
// admitted by the budget before anything is allocated: a handle's bytes are
// planned from its shape and configuration (SIM_Reconstructor::plan_bytes,
// every buffer it can come to hold) and reserved against the budget first;
// while they do not fit, idle handles are deleted least recently used first,
// and when none is idle the request waits until a busy handle is released.
// The handles' reserved bytes therefore never exceed the budget.  A request
// whose handle alone exceeds the budget fails with an error.
#include "server.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <stdexcept>

#include "reconstructor.h"

namespace simrecon {

namespace {
double now_s()
{
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
}  // namespace

ReconServer::ReconServer(int workers, size_t hbm_budget) : budget_(hbm_budget)
{
  // the workers run on the device that is current where the server is made
  if (cudaGetDevice(&device_) != cudaSuccess) device_ = 0;
  if (workers < 1) workers = 1;
  for (int i = 0; i < workers; ++i) workers_.emplace_back([this] { worker_loop(); });
}

ReconServer::~ReconServer()
{
  {
    std::lock_guard<std::mutex> lk(mu_);
    stop_ = true;
  }
  cv_work_.notify_all();
  for (auto& t : workers_) t.join();
  for (auto& h : handles_) delete h->sr;
}

int ReconServer::add_config(const std::string& config_path)
{
  std::lock_guard<std::mutex> lk(mu_);
  configs_.push_back(config_path);
  cstate_.emplace_back();
  return (int)configs_.size() - 1;
}

long long ReconServer::submit(int config, int nx, int ny, int nimages, const void* raw, bool u16, float* out,
                              std::string* err)
{
  if (!raw || !out || nx < 1 || ny < 1 || nimages < 1) {
    *err = "submit: invalid request";
    return -1;
  }
  {
    std::lock_guard<std::mutex> lk(mu_);
    if (config < 0 || config >= (int)configs_.size()) {
      *err = "submit: unknown configuration";
      return -1;
    }
  }
  return enqueue(Request{0, Key{config, nx, ny, nimages}, {raw}, u16, {out}, now_s()});
}

long long ReconServer::enqueue(Request r)
{
  std::lock_guard<std::mutex> lk(mu_);
  r.ticket = next_ticket_++;
  done_[r.ticket] = Done{};
  const long long t = r.ticket;
  queue_.push_back(std::move(r));
  cv_work_.notify_one();
  return t;
}

std::vector<std::vector<size_t>> plan_batch(const std::vector<ReconServer::BatchItem>& items, size_t workers)
{
  // group by (config, shape, input type); a group keeps the caller's order
  std::map<std::tuple<int, int, int, int, bool>, std::vector<size_t>> groups;
  for (size_t i = 0; i < items.size(); ++i) {
    const ReconServer::BatchItem& it = items[i];
    groups[{it.config, it.nx, it.ny, it.nimages, it.u16}].push_back(i);
  }
  // chunks: a group of g items is cut into about one chunk per worker, at
  // most kMaxChunk items each (a chunk holds one handle for its whole run);
  // groups of up to four items stay one chunk (one handle, copies overlapped)
  constexpr size_t kMaxChunk = 16;
  const size_t nw = std::max<size_t>(1, workers);
  struct Group {
    std::vector<std::vector<size_t>> chunks;
    double cost = 0;
  };
  std::vector<Group> order;
  for (auto& [gk, idx] : groups) {
    const size_t per = std::min(kMaxChunk, std::max((idx.size() + nw - 1) / nw, std::min<size_t>(idx.size(), 4)));
    Group g;
    for (size_t a = 0; a < idx.size(); a += per) {
      g.chunks.emplace_back(idx.begin() + a, idx.begin() + std::min(idx.size(), a + per));
      g.cost += (double)std::get<1>(gk) * std::get<2>(gk) * std::get<3>(gk) * g.chunks.back().size();
    }
    order.push_back(std::move(g));
  }
  // groups largest first (the last to start are short), each group's chunks
  // together: a finished group's handles become the least recently used, so
  // under a tight budget they are the ones deleted for the next group's
  std::stable_sort(order.begin(), order.end(), [](const Group& a, const Group& b) { return a.cost > b.cost; });
  std::vector<std::vector<size_t>> chunks;
  for (auto& g : order)
    for (auto& c : g.chunks) chunks.push_back(std::move(c));
  return chunks;
}

int ReconServer::run_batch(const std::vector<BatchItem>& items, std::string* err)
{
  {
    std::lock_guard<std::mutex> lk(mu_);
    for (size_t i = 0; i < items.size(); ++i) {
      const BatchItem& it = items[i];
      if (!it.raw || !it.out || it.nx < 1 || it.ny < 1 || it.nimages < 1 || it.config < 0 ||
          it.config >= (int)configs_.size()) {
        *err = "runBatch: invalid item " + std::to_string(i);
        return -1;
      }
    }
  }
  std::vector<long long> tickets;
  for (const auto& c : plan_batch(items, workers_.size())) {
    const BatchItem& f = items[c[0]];
    Request r{0, Key{f.config, f.nx, f.ny, f.nimages}, {}, f.u16, {}, now_s()};
    for (size_t i : c) {
      r.raws.push_back(items[i].raw);
      r.outs.push_back(items[i].out);
    }
    tickets.push_back(enqueue(std::move(r)));
  }
  int rc = 0;
  for (long long t : tickets) {
    std::string e;
    if (wait(t, nullptr, &e) != 0 && rc == 0) {
      rc = -1;
      *err = e;
    }
  }
  return rc;
}

int ReconServer::wait(long long ticket, double* latency_ms, std::string* err)
{
  std::unique_lock<std::mutex> lk(mu_);
  if (done_.find(ticket) == done_.end()) {
    *err = "wait: unknown ticket";
    return -1;
  }
  // each ticket is waited for once: a second waiter of the same ticket (whose
  // entry the first one erases) gets an error instead of blocking forever
  bool gone = false;
  cv_done_.wait(lk, [&] {
    auto it = done_.find(ticket);
    gone = it == done_.end();
    return gone || it->second.done;
  });
  if (gone) {
    *err = "wait: ticket already waited for";
    return -1;
  }
  Done d = done_[ticket];
  done_.erase(ticket);
  if (latency_ms) *latency_ms = d.latency_ms;
  if (d.rc != 0) *err = d.err;
  return d.rc;
}

int ReconServer::reserve(int config, int nx, int ny, int nimages, int count, std::string* err)
{
  {
    std::lock_guard<std::mutex> lk(mu_);
    if (config < 0 || config >= (int)configs_.size()) {
      *err = "reserve: unknown configuration";
      return -1;
    }
  }
  const Key k{config, nx, ny, nimages};
  std::vector<Handle*> got;
  for (int i = 0; i < count; ++i) {
    // hold the handles taken so far busy, so that each round makes a new one;
    // never wait for memory here (the handles this call holds would not be
    // released while it waits)
    Handle* h = acquire(k, err, false);
    if (!h) break;
    got.push_back(h);
  }
  for (auto* h : got) release(h);
  return (int)got.size();
}

int ReconServer::set_k0_reuse(int config, bool on, std::string* err)
{
  std::lock_guard<std::mutex> lk(mu_);
  if (config < 0 || config >= (int)configs_.size()) {
    *err = "setK0Reuse: unknown configuration";
    return -1;
  }
  cstate_[config].reuse_k0 = on;
  cstate_[config].k0.clear();
  return 0;
}

bool ReconServer::recorded_k0(int config, std::vector<float>* k0)
{
  std::lock_guard<std::mutex> lk(mu_);
  if (config < 0 || config >= (int)configs_.size() || cstate_[config].k0.empty()) return false;
  *k0 = cstate_[config].k0;
  return true;
}

size_t ReconServer::device_bytes_in_use()
{
  std::lock_guard<std::mutex> lk(mu_);
  return in_use_;
}

void ReconServer::counters(long long* created, long long* evicted, long long* admission_waits)
{
  std::lock_guard<std::mutex> lk(mu_);
  if (created) *created = created_;
  if (evicted) *evicted = evicted_;
  if (admission_waits) *admission_waits = admission_waits_;
}

size_t ReconServer::device_bytes_held()
{
  size_t r, h;
  memory_snapshot(&r, &h);
  return h;
}

void ReconServer::memory_snapshot(size_t* reserved, size_t* held)
{
  std::lock_guard<std::mutex> lk(mu_);
  size_t n = 0;
  for (auto& h : handles_) n += h->sr->device_bytes();
  *reserved = in_use_;
  *held = n;
}

int ReconServer::device() const { return device_; }

bool ReconServer::planned_bytes(int config, int nx, int ny, int nimages, size_t* bytes, std::string* err)
{
  const Key k{config, nx, ny, nimages};
  std::string cfg;
  {
    std::lock_guard<std::mutex> lk(mu_);
    if (config < 0 || config >= (int)configs_.size()) {
      *err = "plannedBytes: unknown configuration";
      return false;
    }
    auto it = planned_.find(k);
    if (it != planned_.end()) {
      *bytes = it->second;
      return true;
    }
    cfg = configs_[config];
  }
  if (!SIM_Reconstructor::plan_bytes(nx, ny, nimages, cfg, bytes, err)) return false;
  std::lock_guard<std::mutex> lk(mu_);
  planned_[k] = *bytes;
  return true;
}

ReconServer::Handle* ReconServer::acquire(const Key& k, std::string* err, bool wait_for_memory)
{
  std::string cfg;
  size_t need = 0;
  {
    std::lock_guard<std::mutex> lk(mu_);
    for (auto& h : handles_)
      if (!h->busy && h->key == k) {
        h->busy = true;
        return h.get();
      }
    cfg = configs_[std::get<0>(k)];
    auto it = planned_.find(k);
    if (it != planned_.end()) need = it->second;
  }
  if (!need) {
    if (!SIM_Reconstructor::plan_bytes(std::get<1>(k), std::get<2>(k), std::get<3>(k), cfg, &need, err))
      return nullptr;
    std::lock_guard<std::mutex> lk(mu_);
    planned_[k] = need;
  }
  if (need > budget_) {
    *err = "request needs " + std::to_string(need >> 20) + " MiB of device memory, more than the server's budget";
    return nullptr;
  }
  // admission: reserve `need` bytes within the budget, deleting idle handles
  // (least recently used first) or waiting for busy ones to be released
  for (;;) {
    SIM_Reconstructor* doomed = nullptr;
    {
      std::unique_lock<std::mutex> lk(mu_);
      for (auto& h : handles_)  // a handle of this shape may have been released meanwhile
        if (!h->busy && h->key == k) {
          h->busy = true;
          return h.get();
        }
      if (in_use_ + need <= budget_) {
        in_use_ += need;
        break;
      }
      Handle* lru = nullptr;
      size_t idx = 0;
      for (size_t i = 0; i < handles_.size(); ++i)
        if (!handles_[i]->busy && (!lru || handles_[i]->last_used < lru->last_used)) {
          lru = handles_[i].get();
          idx = i;
        }
      if (lru) {
        in_use_ -= lru->bytes;
        ++evicted_;
        doomed = lru->sr;
        handles_.erase(handles_.begin() + idx);
      } else if (!wait_for_memory) {
        *err = "the server's device-memory budget is taken by busy handles";
        return nullptr;
      } else {
        ++admission_waits_;
        cv_release_.wait(lk);
        continue;
      }
    }
    delete doomed;  // outside the lock: frees device memory
  }
  std::string e1;
  SIM_Reconstructor* sr = SIM_Reconstructor::from_shape(std::get<1>(k), std::get<2>(k), std::get<3>(k), cfg, &e1);
  if (!sr) {
    std::lock_guard<std::mutex> lk(mu_);
    in_use_ -= need;
    cv_release_.notify_all();
    *err = e1;
    return nullptr;
  }
  auto h = std::make_unique<Handle>();
  h->key = k;
  h->sr = sr;
  h->busy = true;
  h->bytes = need;
  Handle* raw = h.get();
  std::lock_guard<std::mutex> lk(mu_);
  ++created_;
  handles_.push_back(std::move(h));
  return raw;
}

void ReconServer::release(Handle* h)
{
  {
    std::lock_guard<std::mutex> lk(mu_);
    h->busy = false;
    h->last_used = now_s();
  }
  cv_release_.notify_all();
}

void ReconServer::worker_loop()
{
  cudaSetDevice(device_);
  for (;;) {
    Request r;
    {
      std::unique_lock<std::mutex> lk(mu_);
      cv_work_.wait(lk, [&] { return stop_ || !queue_.empty(); });
      if (queue_.empty()) return;  // stopping, and every queued request is done
      r = queue_.front();
      queue_.pop_front();
    }
    std::string err;
    int rc = 0;
    Handle* h = acquire(r.key, &err);
    if (!h) {
      rc = -1;
    } else {
      try {
        const int nx = std::get<1>(r.key), ny = std::get<2>(r.key), ni = std::get<3>(r.key);
        const int cfg = std::get<0>(r.key);
        bool reuse = false, record = false;
        std::vector<float> k0;
        {
          std::lock_guard<std::mutex> lk(mu_);
          reuse = cstate_[cfg].reuse_k0 && !cstate_[cfg].k0.empty();
          record = cstate_[cfg].reuse_k0 && cstate_[cfg].k0.empty();
          if (reuse) k0 = cstate_[cfg].k0;
        }
        if (r.raws.size() == 1) {  // the plain per-volume flow
          if (r.u16) h->sr->set_raw_u16((const uint16_t*)r.raws[0], nx, ny, ni);
          else h->sr->set_raw_float((const float*)r.raws[0], nx, ny, ni);
          h->sr->load_and_rescale(0, 0);
          if (reuse) {  // a later time point: the recorded k0, modamps fitted
            h->sr->set_fitted_k0(k0.data());
            if (h->sr->ntimes() < 2) h->sr->set_ntimes(2);
            h->sr->set_cur_time(1);
          } else {
            h->sr->set_cur_time(0);
          }
          h->sr->process_one_volume();
          h->sr->get_result(r.outs[0]);
          if (record) {
            std::vector<float> fk(2 * kMaxDirs);
            h->sr->get_fit(fk.data(), nullptr);
            std::lock_guard<std::mutex> lk(mu_);
            if (cstate_[cfg].reuse_k0 && cstate_[cfg].k0.empty()) cstate_[cfg].k0 = fk;
          }
        } else {
          h->sr->process_series(r.raws.data(), r.u16, r.outs.data(), (int)r.raws.size(), 0, true);
        }
      } catch (const std::exception& e) {
        rc = -1;
        err = e.what();
      }
      release(h);
    }
    const double t = now_s();
    {
      std::lock_guard<std::mutex> lk(mu_);
      Done& d = done_[r.ticket];
      d.done = true;
      d.rc = rc;
      d.err = err;
      d.latency_ms = (t - r.t_submit) * 1e3;
    }
    cv_done_.notify_all();
  }
}

}  // namespace simrecon
