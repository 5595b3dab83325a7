// Stand-in for the un-vendored TBB submodule: the film merge and the block
// generator only need tbb::mutex with a scoped lock (std::mutex underneath).
#pragma once
#include <cstring>
#include <mutex>
namespace tbb {
struct mutex {
    std::mutex m;
    void lock() { m.lock(); }
    void unlock() { m.unlock(); }
    struct scoped_lock {
        mutex& r;
        explicit scoped_lock(mutex& x) : r(x) { r.lock(); }
        ~scoped_lock() { r.unlock(); }
    };
};
}  // namespace tbb
