// A persistent pool of host threads for the library's host-side work that
// splits into independent items (the ghost programs' emission after a
// regrid).  Threads are created once, on first use, and wait on a condition
// variable between calls; parallel_for(n, f) runs f(0..n-1) on them and on
// the calling thread and returns when every item is done.  A call made while
// another is running (another host thread, or an item calling parallel_for)
// runs its items on the calling thread alone, so calls never wait for each
// other.
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include "hier.h"

namespace bsamg {

namespace {

class Pool {
 public:
  Pool() {
    unsigned n = std::max(1u, std::thread::hardware_concurrency());
    for (unsigned t = 1; t < n; t++) workers_.emplace_back([this] { loop(); });
  }
  ~Pool() {
    {
      std::lock_guard<std::mutex> g(mu_);
      quit_ = true;
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
  }
  void run(int n, const std::function<void(int)>& f) {
    std::unique_lock<std::mutex> busy(run_mu_, std::try_to_lock);
    if (!busy.owns_lock() || workers_.empty() || n < 2) {
      for (int x = 0; x < n; x++) f(x);
      return;
    }
    {
      std::lock_guard<std::mutex> g(mu_);
      fn_ = &f;
      n_ = n;
      next_.store(0);
      left_ = n;
      gen_++;
    }
    cv_.notify_all();
    work();
    std::unique_lock<std::mutex> g(mu_);
    done_.wait(g, [&] { return left_ == 0; });
    fn_ = nullptr;
  }

 private:
  void work() {
    int done = 0;
    for (int x; (x = next_.fetch_add(1)) < n_;) {
      (*fn_)(x);
      done++;
    }
    if (done) {
      std::lock_guard<std::mutex> g(mu_);
      left_ -= done;
      if (left_ == 0) done_.notify_all();
    }
  }
  void loop() {
    unsigned long long seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> g(mu_);
        cv_.wait(g, [&] { return quit_ || (gen_ != seen && fn_); });
        if (quit_) return;
        seen = gen_;
      }
      work();
    }
  }
  std::vector<std::thread> workers_;
  std::mutex mu_, run_mu_;
  std::condition_variable cv_, done_;
  const std::function<void(int)>* fn_ = nullptr;
  int n_ = 0, left_ = 0;
  std::atomic<int> next_{0};
  unsigned long long gen_ = 0;
  bool quit_ = false;
};

}  // namespace

void parallel_for(int n, const std::function<void(int)>& f) {
  static Pool pool;
  pool.run(n, f);
}

}  // namespace bsamg
