// Request server over pooled reconstructor handles (the serving form of the
// SR_* flow): volumes of different shapes and acquisition configurations are
// submitted from any thread, run concurrently by worker threads that each
// drive their own handle (own CUDA stream), and waited for by ticket.
#pragma once
#include <condition_variable>
#include <cstddef>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

class SIM_Reconstructor;

namespace simrecon {

class ReconServer {
 public:
  // workers: concurrent volumes; hbm_budget: device bytes the handles may hold
  ReconServer(int workers, size_t hbm_budget);
  ~ReconServer();
  // an acquisition configuration: a reference-style config file naming its OTF
  int add_config(const std::string& config_path);
  // one volume (the SR_setRaw layout) -> out (the SR_getResult layout); the
  // buffers stay the caller's and must stay valid until wait() returns.
  // Processed like a volume at time 0 (k0 fitted).  Returns a ticket, or -1.
  long long submit(int config, int nx, int ny, int nimages, const void* raw, bool u16, float* out,
                   std::string* err);
  // blocks until the request is done; latency = submission to result in
  // host memory.  Returns 0, or -1 with the request's error.
  int wait(long long ticket, double* latency_ms, std::string* err);
  // k0 reuse per configuration (off by default): the first request of the
  // configuration to finish searches k0 as usual and records it; every later
  // request of that configuration is processed like a later time point of a
  // series (the recorded k0 reused, modamps fitted, bleach correction against
  // its own planes), whatever its shape.  Turning it on clears the record.
  int set_k0_reuse(int config, bool on, std::string* err);
  // the recorded k0 of a configuration (2 floats per direction); false if none
  bool recorded_k0(int config, std::vector<float>* k0);
  // device bytes reserved against the budget by the pooled handles (each
  // handle's planned maximum); never above the budget
  size_t device_bytes_in_use();
  // device bytes the pooled handles actually hold now (at most the reserved)
  size_t device_bytes_held();
  // both under one lock: a consistent pair (held <= reserved)
  void memory_snapshot(size_t* reserved, size_t* held);
  // handles created and deleted (budget evictions) since construction, and
  // how often a request waited for device memory to be released
  void counters(long long* created, long long* evicted, long long* admission_waits = nullptr);
  int device() const;
  // planned device bytes of a handle for this configuration and shape (what
  // admission reserves for it); false with the error if it cannot be planned
  bool planned_bytes(int config, int nx, int ny, int nimages, size_t* bytes, std::string* err);
  // create handles for a shape up front so that the first requests of that
  // shape do not pay for their creation; returns how many were created
  int reserve(int config, int nx, int ny, int nimages, int count, std::string* err);

  // A batch of standalone acquisitions of uneven shapes (every item processed
  // like a submit()ted volume).  Items are grouped by (config, shape); each
  // group is cut into chunks that a worker runs back to back on one handle
  // with the upload of the next item and the download of the previous one
  // overlapped with the computation (SIM_Reconstructor::process_series in its
  // standalone form), and the workers run chunks of different shapes
  // concurrently, groups largest first with each group's chunks together.
  // Blocks until every item is done; returns 0, or -1 with the first failing
  // item's error.
  struct BatchItem {
    int config, nx, ny, nimages;
    const void* raw;
    bool u16;
    float* out;
  };
  int run_batch(const std::vector<BatchItem>& items, std::string* err);

 private:
  using Key = std::tuple<int, int, int, int>;  // config, nx, ny, nimages
  struct Request {
    long long ticket;
    Key key;
    std::vector<const void*> raws;  // one volume, or a chunk of a batch
    bool u16;
    std::vector<float*> outs;
    double t_submit;
  };
  struct Done {
    bool done = false;
    int rc = 0;
    std::string err;
    double latency_ms = 0;
  };
  struct Handle {
    Key key;
    SIM_Reconstructor* sr = nullptr;
    bool busy = false;
    double last_used = 0;
    size_t bytes = 0;
  };
  void worker_loop();
  Handle* acquire(const Key& k, std::string* err, bool wait_for_memory = true);
  long long enqueue(Request r);
  void release(Handle* h);

  std::vector<std::string> configs_;
  struct ConfigState {
    bool reuse_k0 = false;
    std::vector<float> k0;  // empty until recorded
  };
  std::vector<ConfigState> cstate_;
  std::mutex mu_;
  std::condition_variable cv_work_, cv_done_, cv_release_;
  std::deque<Request> queue_;
  std::map<long long, Done> done_;
  std::vector<std::unique_ptr<Handle>> handles_;
  size_t budget_, in_use_ = 0;
  std::map<Key, size_t> planned_;  // planned device bytes per (configuration, shape)
  int device_ = 0;
  long long next_ticket_ = 1;
  long long created_ = 0, evicted_ = 0, admission_waits_ = 0;
  bool stop_ = false;
  std::vector<std::thread> workers_;
};

// The batch schedule run_batch uses: the items grouped by (config, nx, ny,
// nimages, input type), each group cut into chunks (about one per worker, at
// most 16 items, groups of up to four items whole), groups ordered by
// nx * ny * nimages * items, largest first, each group's chunks together.
// Returns the chunks in execution order, each a list of item indices in the
// caller's order.
std::vector<std::vector<size_t>> plan_batch(const std::vector<ReconServer::BatchItem>& items, size_t workers);

}  // namespace simrecon
