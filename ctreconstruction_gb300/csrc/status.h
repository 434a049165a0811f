// Per-thread last-error state behind ctgb_last_error().
#pragma once
#include "../../include/ctgb.h"

namespace ctgb {
int set_error(int status, const char *fmt, ...);   // records the message, returns status
void clear_error();
int last_status();
}  // namespace ctgb
