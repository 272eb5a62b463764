// Internal declarations shared by the host-side translation units.
#ifndef MCLICKS_HOST_INTERNAL_H
#define MCLICKS_HOST_INTERNAL_H

#include <cstdint>
#include <string>
#include <vector>

#include "mclicks.h"

namespace mch {

// Records msg as the calling thread's last error and returns code.
int set_error(int code, const std::string& msg);

// One set of sessions, structure of arrays; docs and pidx session-major.
struct SessionSet {
    std::vector<int32_t> query;
    std::vector<int32_t> docs;    // n * 10
    std::vector<int32_t> pidx;    // n * 10
    std::vector<uint16_t> click;  // n, bit r = click at rank r
    int64_t size() const { return (int64_t)query.size(); }
};

}  // namespace mch

struct mc_dataset {
    mch::SessionSet train, test;
    int64_t n_qd = 0;
};

#endif  // MCLICKS_HOST_INTERNAL_H
