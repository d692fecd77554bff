/* Thread-pool stand-in for the parts of Intel TBB 4.2 that the reference
 * renderer uses: atomic, blocked_range, parallel_for, pipeline/filter,
 * parallel_invoke, tick_count, enumerable_thread_specific and
 * cache_aligned_allocator.  Oracle build only.
 *
 * It is really parallel (std::thread workers), so the reference's CPU path
 * can be timed on all host cores.  The worker count comes from the
 * SKW_REF_THREADS environment variable, else std::thread::hardware_concurrency.
 *
 * Pipeline semantics: the serial filters of one pipeline share one mutex
 * (so the reference's unsynchronised chunk "available" flags are published
 * between its serial input and serial output filters), parallel filters run
 * concurrently, and at most min(workers, max_tokens) items are in flight. */
#ifndef SKW_REF_SHIM_TBB_H
#define SKW_REF_SHIM_TBB_H

#include <atomic>
#include <chrono>
#include <cstddef>
#include <cstdlib>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

namespace tbb {

inline unsigned shim_num_workers() {
  const char *env = std::getenv("SKW_REF_THREADS");
  if (env && std::atoi(env) > 0) return (unsigned)std::atoi(env);
  unsigned n = std::thread::hardware_concurrency();
  return n ? n : 1;
}

/* Runs fn(worker_index) on `n` threads (the caller is worker 0) and joins. */
inline void shim_run_workers(unsigned n, const std::function<void(unsigned)> &fn) {
  if (n <= 1) {
    fn(0);
    return;
  }
  std::vector<std::thread> threads;
  threads.reserve(n - 1);
  for (unsigned i = 1; i < n; ++i) threads.emplace_back(fn, i);
  fn(0);
  for (auto &t : threads) t.join();
}

template <typename T>
class atomic {
 public:
  atomic() : v_() {}
  operator T() const { return v_.load(); }
  T operator=(T x) {
    v_.store(x);
    return x;
  }
  atomic &operator=(const atomic &o) {
    v_.store(o.v_.load());
    return *this;
  }
  T operator++() { return ++v_; }
  T operator--() { return --v_; }
  T operator++(int) { return v_++; }
  T operator--(int) { return v_--; }
  T operator+=(T x) { return v_ += x; }
  T operator-=(T x) { return v_ -= x; }
  T fetch_and_add(T x) { return v_.fetch_add(x); }
  T fetch_and_increment() { return v_.fetch_add(1); }
  T compare_and_swap(T value, T comparand) {
    v_.compare_exchange_strong(comparand, value);
    return comparand;
  }

 private:
  std::atomic<T> v_;
};

template <typename Value>
class blocked_range {
 public:
  typedef Value const_iterator;
  blocked_range(Value b, Value e, size_t grain = 1) : b_(b), e_(e), grain_(grain ? grain : 1) {}
  Value begin() const { return b_; }
  Value end() const { return e_; }
  size_t size() const { return (size_t)(e_ - b_); }
  size_t grainsize() const { return grain_; }
  bool empty() const { return !(b_ < e_); }

 private:
  Value b_, e_;
  size_t grain_;
};

/* Splits [b, e) into grain-sized pieces handed out dynamically.  Like TBB,
 * every worker runs its own copy of the body (the reference relies on this:
 * IrradiancePhotonProcess keeps per-copy scratch, PhotonInternalTypes.h:262-301). */
template <typename Value, typename Body>
void parallel_for(const blocked_range<Value> &range, const Body &body) {
  size_t total = range.size();
  if (total == 0) return;
  size_t grain = range.grainsize();
  size_t pieces = (total + grain - 1) / grain;
  /* Keep pieces small enough to balance but not smaller than the grain. */
  unsigned workers = shim_num_workers();
  if (pieces <= 1 || workers <= 1) {
    const Body local(body);
    local(range);
    return;
  }
  size_t chunk = grain;
  if (total / (workers * 8) > chunk) chunk = total / (workers * 8);
  std::atomic<size_t> next(0);
  unsigned n = (unsigned)std::min<size_t>(workers, (total + chunk - 1) / chunk);
  shim_run_workers(n, [&](unsigned) {
    const Body local(body);
    for (;;) {
      size_t s = next.fetch_add(chunk);
      if (s >= total) break;
      size_t e = std::min(total, s + chunk);
      local(blocked_range<Value>(range.begin() + (Value)s, range.begin() + (Value)e, grain));
    }
  });
}

template <typename Index, typename Func>
void parallel_for(Index first, Index last, const Func &f) {
  parallel_for(blocked_range<Index>(first, last, 1), [&](const blocked_range<Index> &r) {
    for (Index i = r.begin(); i != r.end(); ++i) f(i);
  });
}

template <typename F0, typename F1>
void parallel_invoke(const F0 &f0, const F1 &f1) {
  std::thread t(f1);
  f0();
  t.join();
}

template <typename F0, typename F1, typename F2>
void parallel_invoke(const F0 &f0, const F1 &f1, const F2 &f2) {
  std::thread t1(f1), t2(f2);
  f0();
  t1.join();
  t2.join();
}

class filter {
 public:
  enum mode { parallel = 0, serial_in_order = 1, serial_out_of_order = 2, serial = serial_in_order };
  explicit filter(mode m) : mode_(m) {}
  explicit filter(bool is_serial) : mode_(is_serial ? serial_in_order : parallel) {}
  virtual ~filter() {}
  virtual void *operator()(void *item) = 0;
  bool is_serial() const { return mode_ != parallel; }

 private:
  mode mode_;
};

class pipeline {
 public:
  void add_filter(filter &f) { filters_.push_back(&f); }
  void clear() { filters_.clear(); }
  void run(size_t max_tokens) {
    if (filters_.empty()) return;
    unsigned n = shim_num_workers();
    if (max_tokens > 0 && n > max_tokens) n = (unsigned)max_tokens;
    std::mutex serial_mutex;
    std::atomic<bool> done(false);
    shim_run_workers(n, [&](unsigned) {
      for (;;) {
        void *item = nullptr;
        {
          std::lock_guard<std::mutex> lock(serial_mutex);
          if (done.load()) return;
          item = (*filters_[0])(nullptr);
          if (!item) {
            done.store(true);
            return;
          }
        }
        for (size_t i = 1; i < filters_.size() && item; ++i) {
          if (filters_[i]->is_serial()) {
            std::lock_guard<std::mutex> lock(serial_mutex);
            item = (*filters_[i])(item);
          } else {
            item = (*filters_[i])(item);
          }
        }
      }
    });
  }

 private:
  std::vector<filter *> filters_;
};

class tick_count {
 public:
  class interval_t {
   public:
    explicit interval_t(double s = 0) : s_(s) {}
    double seconds() const { return s_; }

   private:
    double s_;
  };
  tick_count() : t_() {}
  static tick_count now() {
    tick_count t;
    t.t_ = std::chrono::steady_clock::now();
    return t;
  }
  friend interval_t operator-(const tick_count &a, const tick_count &b) {
    return interval_t(std::chrono::duration<double>(a.t_ - b.t_).count());
  }

 private:
  std::chrono::steady_clock::time_point t_;
};

template <typename T>
class cache_aligned_allocator : public std::allocator<T> {
 public:
  template <typename U>
  struct rebind {
    typedef cache_aligned_allocator<U> other;
  };
  cache_aligned_allocator() {}
  template <typename U>
  cache_aligned_allocator(const cache_aligned_allocator<U> &) {}
};

enum ets_key_usage_type { ets_key_per_instance, ets_no_key };

/* One T per thread, created on first use; local(exists) reports whether it
 * existed before.  A per-thread cache keeps the common path lock-free. */
template <typename T, typename Alloc = cache_aligned_allocator<T>, ets_key_usage_type K = ets_no_key>
class enumerable_thread_specific {
 public:
  enumerable_thread_specific() {}
  T &local() {
    bool e;
    return local(e);
  }
  T &local(bool &exists) {
    thread_local std::map<const void *, T *> cache;
    auto it = cache.find(this);
    if (it != cache.end()) {
      exists = true;
      return *it->second;
    }
    std::lock_guard<std::mutex> lock(mutex_);
    items_.emplace_back(new T());
    T *p = items_.back().get();
    cache[this] = p;
    exists = false;
    return *p;
  }

 private:
  std::mutex mutex_;
  std::vector<std::unique_ptr<T>> items_;
};

}  // namespace tbb

#endif
