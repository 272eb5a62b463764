// Per-thread error status of the C-ABI.
#include <cstring>
#include <string>

#include "host_internal.h"

namespace mch {

static thread_local int g_last_code = MC_OK;
static thread_local std::string g_last_msg;

int set_error(int code, const std::string& msg) {
    g_last_code = code;
    g_last_msg = msg;
    return code;
}

}  // namespace mch

extern "C" int mc_last_error(char* buf, size_t len) {
    if (buf && len) {
        size_t n = mch::g_last_msg.size() < len - 1 ? mch::g_last_msg.size() : len - 1;
        std::memcpy(buf, mch::g_last_msg.data(), n);
        buf[n] = 0;
    }
    return mch::g_last_code;
}

extern "C" const char* mc_version(void) { return "massiveclicks-gb300 0.1.0"; }
