// Internal declarations shared by the host-side translation units.
#ifndef MCLICKS_HOST_INTERNAL_H
#define MCLICKS_HOST_INTERNAL_H

#include <cstdint>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "mclicks.h"

namespace mch {

// Records msg as the calling thread's last error and returns code.
int set_error(int code, const std::string& msg);

// An allocator whose resize leaves new elements uninitialised: the partition
// arrays are sized first and then filled by host threads in parallel, so the
// pages are first touched by those threads rather than zeroed by one.
template <class T>
struct NoInitAlloc : std::allocator<T> {
    template <class U>
    struct rebind {
        using other = NoInitAlloc<U>;
    };
    NoInitAlloc() = default;
    template <class U>
    NoInitAlloc(const NoInitAlloc<U>&) noexcept {}
    template <class U>
    void construct(U* p) noexcept {
        ::new ((void*)p) U;
    }
    template <class U, class... A>
    void construct(U* p, A&&... a) {
        ::new ((void*)p) U(std::forward<A>(a)...);
    }
};
template <class T>
using RawVec = std::vector<T, NoInitAlloc<T>>;

// One set of sessions, structure of arrays; docs and pidx session-major.
struct SessionSet {
    RawVec<int32_t> query;
    RawVec<int32_t> docs;    // n * 10
    RawVec<int32_t> pidx;    // n * 10
    RawVec<uint16_t> click;  // n, bit r = click at rank r
    int64_t size() const { return (int64_t)query.size(); }
};

}  // namespace mch

struct mc_dataset {
    mch::SessionSet train, test;
    int64_t n_qd = 0;
};

#endif  // MCLICKS_HOST_INTERNAL_H
