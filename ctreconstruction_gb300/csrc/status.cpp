#include "status.h"

#include <cstdarg>
#include <cstdio>

namespace ctgb {
static thread_local char g_msg[512] = "";
static thread_local int g_status = CTGB_OK;

int set_error(int status, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(g_msg, sizeof g_msg, fmt, ap);
    va_end(ap);
    g_status = status;
    return status;
}

void clear_error() {
    g_msg[0] = 0;
    g_status = CTGB_OK;
}

int last_status() { return g_status; }
}  // namespace ctgb

extern "C" const char *ctgb_last_error(void) { return ctgb::g_msg; }
extern "C" const char *ctgb_version(void) { return "ctgb 0.1 (sm_103a)"; }
