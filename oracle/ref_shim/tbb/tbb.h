/* ORACLE build support — test infrastructure only.
 *
 * A serial stand-in for the parts of Intel oneTBB that SQUANDER's C++ sources include
 * (parallel_for over blocked_range, parallel_invoke, enumerable_thread_specific,
 * combinable, the mutexes, task_group/task_arena, tick_count and the allocators).
 * Every "parallel" construct runs its body once, in order, on the calling thread, so a
 * reference build against this header is deterministic: reductions happen in index order.
 * TBB contributes threading only, no arithmetic, to the code paths it is used on.
 */
#ifndef SQG_REF_SHIM_TBB_H
#define SQG_REF_SHIM_TBB_H

#include <chrono>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <functional>
#include <malloc.h>
#include <memory>
#include <new>
#include <utility>
#include <vector>

namespace tbb {

template <typename Value>
class blocked_range {
public:
    typedef Value const_iterator;
    typedef std::size_t size_type;
    blocked_range() : lo_(), hi_(), grain_(1) {}
    blocked_range(Value begin, Value end, std::size_t grain = 1) : lo_(begin), hi_(end), grain_(grain) {}
    Value begin() const { return lo_; }
    Value end() const { return hi_; }
    std::size_t size() const { return std::size_t(hi_ - lo_); }
    std::size_t grainsize() const { return grain_; }
    bool empty() const { return !(lo_ < hi_); }
    bool is_divisible() const { return false; }
private:
    Value lo_, hi_;
    std::size_t grain_;
};

class auto_partitioner {};
class simple_partitioner {};
class static_partitioner {};
class affinity_partitioner {};

template <typename Range, typename Body>
void parallel_for(const Range& range, const Body& body) {
    if (!range.empty()) body(range);
}
template <typename Range, typename Body, typename Partitioner>
void parallel_for(const Range& range, const Body& body, Partitioner&) {
    if (!range.empty()) body(range);
}
template <typename Range, typename Body, typename Partitioner>
void parallel_for(const Range& range, const Body& body, const Partitioner&) {
    if (!range.empty()) body(range);
}
template <typename Index, typename Function>
void parallel_for(Index first, Index last, Index step, const Function& f) {
    for (Index i = first; i < last; i += step) f(i);
}
template <typename Index, typename Function>
void parallel_for(Index first, Index last, const Function& f) {
    for (Index i = first; i < last; ++i) f(i);
}

inline void parallel_invoke() {}
template <typename F, typename... Rest>
void parallel_invoke(const F& f, const Rest&... rest) {
    f();
    parallel_invoke(rest...);
}

template <typename T>
class enumerable_thread_specific {
public:
    typedef typename std::deque<T>::iterator iterator;
    typedef typename std::deque<T>::const_iterator const_iterator;
    enumerable_thread_specific() : init_([]() { return T(); }) {}
    template <typename F, typename = decltype(std::declval<F>()())>
    explicit enumerable_thread_specific(F f) : init_(f) {}
    explicit enumerable_thread_specific(const T& exemplar) : init_([exemplar]() { return exemplar; }) {}
    T& local() {
        if (slot_.empty()) slot_.push_back(init_());
        return slot_.front();
    }
    T& local(bool& exists) {
        exists = !slot_.empty();
        return local();
    }
    iterator begin() { return slot_.begin(); }
    iterator end() { return slot_.end(); }
    const_iterator begin() const { return slot_.begin(); }
    const_iterator end() const { return slot_.end(); }
    std::size_t size() const { return slot_.size(); }
    bool empty() const { return slot_.empty(); }
    void clear() { slot_.clear(); }
    template <typename Op>
    T combine(Op op) {
        if (slot_.empty()) return init_();
        T acc = slot_.front();
        for (std::size_t i = 1; i < slot_.size(); ++i) acc = op(acc, slot_[i]);
        return acc;
    }
    template <typename F>
    void combine_each(F f) {
        for (auto& v : slot_) f(v);
    }
private:
    std::function<T()> init_;
    std::deque<T> slot_;
};

template <typename T>
class combinable {
public:
    combinable() : ets_() {}
    template <typename F>
    explicit combinable(F f) : ets_(f) {}
    T& local() { return ets_.local(); }
    T& local(bool& exists) { return ets_.local(exists); }
    void clear() { ets_.clear(); }
    template <typename Op>
    T combine(Op op) { return ets_.combine(op); }
    template <typename F>
    void combine_each(F f) { ets_.combine_each(f); }
private:
    enumerable_thread_specific<T> ets_;
};

/* Mutexes: the serial stand-in never contends, so locking is a no-op. */
#define SQG_SHIM_MUTEX(NAME)                                                  \
    class NAME {                                                              \
    public:                                                                   \
        class scoped_lock {                                                   \
        public:                                                               \
            scoped_lock() {}                                                  \
            explicit scoped_lock(NAME&) {}                                    \
            scoped_lock(NAME&, bool) {}                                       \
            void acquire(NAME&) {}                                            \
            void acquire(NAME&, bool) {}                                      \
            bool try_acquire(NAME&) { return true; }                          \
            bool try_acquire(NAME&, bool) { return true; }                    \
            void release() {}                                                 \
            bool upgrade_to_writer() { return true; }                         \
            bool downgrade_to_reader() { return true; }                       \
        };                                                                    \
        void lock() {}                                                        \
        void unlock() {}                                                      \
        bool try_lock() { return true; }                                      \
    };
SQG_SHIM_MUTEX(spin_mutex)
SQG_SHIM_MUTEX(queuing_mutex)
SQG_SHIM_MUTEX(queuing_rw_mutex)
SQG_SHIM_MUTEX(spin_rw_mutex)
SQG_SHIM_MUTEX(mutex)
#undef SQG_SHIM_MUTEX

class task_group {
public:
    template <typename F>
    void run(const F& f) { f(); }
    template <typename F>
    void run_and_wait(const F& f) { f(); }
    void wait() {}
};

class task_arena {
public:
    task_arena(int = -1, unsigned = 1) {}
    template <typename F>
    auto execute(const F& f) -> decltype(f()) { return f(); }
    void initialize() {}
    void initialize(int) {}
};

class global_control {
public:
    enum parameter { max_allowed_parallelism, thread_stack_size };
    global_control(parameter, std::size_t) {}
    static std::size_t active_value(parameter) { return 1; }
};

namespace this_task_arena {
inline int max_concurrency() { return 1; }
}

class tick_count {
public:
    class interval_t {
    public:
        interval_t() : s_(0.0) {}
        explicit interval_t(double s) : s_(s) {}
        double seconds() const { return s_; }
        interval_t& operator+=(const interval_t& o) { s_ += o.s_; return *this; }
        interval_t operator+(const interval_t& o) const { return interval_t(s_ + o.s_); }
    private:
        double s_;
    };
    tick_count() : t_(0.0) {}
    static tick_count now() {
        tick_count t;
        t.t_ = std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
        return t;
    }
    interval_t operator-(const tick_count& o) const { return interval_t(t_ - o.t_); }
private:
    double t_;
};

template <typename T>
class cache_aligned_allocator : public std::allocator<T> {
public:
    template <typename U>
    struct rebind { typedef cache_aligned_allocator<U> other; };
    cache_aligned_allocator() noexcept {}
    template <typename U>
    cache_aligned_allocator(const cache_aligned_allocator<U>&) noexcept {}
};

template <typename T>
class scalable_allocator : public std::allocator<T> {
public:
    template <typename U>
    struct rebind { typedef scalable_allocator<U> other; };
    scalable_allocator() noexcept {}
    template <typename U>
    scalable_allocator(const scalable_allocator<U>&) noexcept {}
};

}  // namespace tbb

/* scalable_allocator.h C interface: aligned allocations through posix_memalign. */
inline void* scalable_aligned_malloc(std::size_t size, std::size_t alignment) {
    void* p = nullptr;
    if (alignment < sizeof(void*)) alignment = sizeof(void*);
    if (posix_memalign(&p, alignment, size ? size : 1) != 0) return nullptr;
    return p;
}
inline void scalable_aligned_free(void* p) { std::free(p); }
inline void* scalable_aligned_realloc(void* p, std::size_t size, std::size_t alignment) {
    if (p == nullptr) return scalable_aligned_malloc(size, alignment);
    void* q = scalable_aligned_malloc(size, alignment);
    if (q == nullptr) return nullptr;
    /* keep the contents up to the smaller of the two sizes, as realloc does */
    std::size_t old = malloc_usable_size(p);
    std::memcpy(q, p, old < size ? old : size);
    std::free(p);
    return q;
}
inline void* scalable_malloc(std::size_t size) { return std::malloc(size ? size : 1); }
inline void scalable_free(void* p) { std::free(p); }

#endif
