#include "parallel.h"

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdlib>
#include <exception>
#include <mutex>
#include <thread>
#include <unistd.h>
#include <vector>

namespace bgpu {

namespace {

thread_local bool t_in_pool = false;

class Pool {
 public:
  explicit Pool(int n) {
    for (int i = 0; i < n - 1; ++i) workers_.emplace_back([this] { loop(); });
  }
  ~Pool() {
    {
      std::lock_guard<std::mutex> g(m_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
  }

  void run(int n, const std::function<void(int)>& fn) {
    std::lock_guard<std::mutex> one(run_m_);  // one loop at a time
    {
      std::lock_guard<std::mutex> g(m_);
      fn_ = &fn;
      n_ = n;
      next_.store(0);
      active_ = (int)workers_.size();
      err_ = nullptr;
      ++gen_;
    }
    cv_.notify_all();
    t_in_pool = true;
    work();
    t_in_pool = false;
    std::unique_lock<std::mutex> g(m_);
    done_cv_.wait(g, [this] { return active_ == 0; });
    fn_ = nullptr;
    if (err_) std::rethrow_exception(err_);
  }

 private:
  void work() {
    for (;;) {
      const int i = next_.fetch_add(1);
      if (i >= n_) break;
      try {
        (*fn_)(i);
      } catch (...) {
        std::lock_guard<std::mutex> g(m_);
        if (!err_) err_ = std::current_exception();
        next_.store(n_);
      }
    }
  }
  void loop() {
    t_in_pool = true;
    long seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> g(m_);
        cv_.wait(g, [&] { return stop_ || gen_ != seen; });
        if (stop_) return;
        seen = gen_;
      }
      work();
      {
        std::lock_guard<std::mutex> g(m_);
        if (--active_ == 0) done_cv_.notify_all();
      }
    }
  }

  std::vector<std::thread> workers_;
  std::mutex m_, run_m_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(int)>* fn_ = nullptr;
  int n_ = 0;
  std::atomic<int> next_{0};
  int active_ = 0;
  long gen_ = 0;
  bool stop_ = false;
  std::exception_ptr err_;
};

Pool& pool() {
  static Pool p(host_threads());
  return p;
}

// the pool's threads do not exist in a forked child
const pid_t g_pool_pid = getpid();

}  // namespace

int host_threads() {
  static const int n = [] {
    if (const char* e = std::getenv("BGPU_HOST_THREADS")) {
      const int v = std::atoi(e);
      if (v > 0) return v;
    }
    return std::max(1, std::min(32, (int)std::thread::hardware_concurrency()));
  }();
  return n;
}

void parallel_for(int n, const std::function<void(int)>& fn) {
  if (n <= 0) return;
  if (t_in_pool || n == 1 || host_threads() == 1 || getpid() != g_pool_pid) {
    for (int i = 0; i < n; ++i) fn(i);
    return;
  }
  pool().run(n, fn);
}

}  // namespace bgpu
