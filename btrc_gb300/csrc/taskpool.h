// A small fork-join task pool for the host-side scene build: worker threads take tasks
// from one shared queue, and a thread waiting for a group of tasks runs queued tasks
// itself until the group is done, so nested fork-join (a task that spawns and waits
// for subtasks) never deadlocks.
#pragma once

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstddef>
#include <deque>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace bt {

class TaskPool;

// The pool the calling thread works for: set on the pool's workers and, through
// PoolScope, on a thread that waits on it, so that code running inside a task (a scene
// load or build in a batch) reuses that pool instead of starting threads of its own.
inline TaskPool *&current_pool()
{
    thread_local TaskPool *p = nullptr;
    return p;
}

class TaskPool
{
public:
    struct Group
    {
        std::atomic<int> pending{ 0 };
    };

    // threads: total threads working on the pool's tasks, the caller included
    explicit TaskPool(int threads)
    {
        const int n = std::max(1, threads) - 1;
        for(int k = 0; k < n; ++k)
            workers_.emplace_back([this] { work(); });
    }

    ~TaskPool()
    {
        {
            std::lock_guard<std::mutex> lock(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for(auto &t : workers_)
            t.join();
    }

    TaskPool(const TaskPool &) = delete;
    TaskPool &operator=(const TaskPool &) = delete;

    int threads() const { return static_cast<int>(workers_.size()) + 1; }

    void run(Group &g, std::function<void()> fn)
    {
        g.pending.fetch_add(1, std::memory_order_relaxed);
        {
            std::lock_guard<std::mutex> lock(mu_);
            queue_.push_back({ &g, std::move(fn) });
        }
        cv_.notify_one();
    }

    // run queued tasks on this thread until every task of g has finished
    void wait(Group &g)
    {
        while(g.pending.load(std::memory_order_acquire) > 0)
        {
            Task t;
            {
                std::unique_lock<std::mutex> lock(mu_);
                if(queue_.empty())
                {
                    lock.unlock();
                    std::this_thread::yield();
                    continue;
                }
                t = std::move(queue_.back());
                queue_.pop_back();
            }
            execute(t);
        }
    }

    // fn(begin, end) over [0, n) in about `chunks` pieces, in parallel; returns when done
    template<class F>
    void parallel_for(size_t n, size_t min_chunk, F &&fn)
    {
        if(n == 0)
            return;
        const size_t pieces = std::max<size_t>(1, std::min<size_t>(n / std::max<size_t>(min_chunk, 1),
                                                                   static_cast<size_t>(threads()) * 4));
        if(pieces <= 1)
        {
            fn(size_t(0), n);
            return;
        }
        Group g;
        const size_t step = (n + pieces - 1) / pieces;
        for(size_t b = step; b < n; b += step)
        {
            const size_t e = std::min(n, b + step);
            run(g, [&fn, b, e] { fn(b, e); });
        }
        fn(size_t(0), std::min(n, step));
        wait(g);
    }

private:
    struct Task
    {
        Group *group = nullptr;
        std::function<void()> fn;
    };

    void execute(Task &t)
    {
        t.fn();
        t.group->pending.fetch_sub(1, std::memory_order_acq_rel);
    }

    void work()
    {
        current_pool() = this;
        for(;;)
        {
            Task t;
            {
                std::unique_lock<std::mutex> lock(mu_);
                cv_.wait(lock, [this] { return stop_ || !queue_.empty(); });
                if(stop_ && queue_.empty())
                    return;
                // oldest first: the largest subtrees were queued first
                t = std::move(queue_.front());
                queue_.pop_front();
            }
            execute(t);
        }
    }

    std::mutex mu_;
    std::condition_variable cv_;
    std::deque<Task> queue_;
    std::vector<std::thread> workers_;
    bool stop_ = false;
};

// marks the calling thread as working for `pool` while the scope lives
class PoolScope
{
public:
    explicit PoolScope(TaskPool &pool) : prev_(current_pool()) { current_pool() = &pool; }
    ~PoolScope() { current_pool() = prev_; }
    PoolScope(const PoolScope &) = delete;
    PoolScope &operator=(const PoolScope &) = delete;

private:
    TaskPool *prev_;
};

// f(pool) on the pool the thread already works for, or on a new pool of `threads`
template<class F>
void with_pool(int threads, F &&f)
{
    if(TaskPool *p = current_pool())
    {
        f(*p);
        return;
    }
    TaskPool pool(threads);
    PoolScope scope(pool);
    f(pool);
}

} // namespace bt
