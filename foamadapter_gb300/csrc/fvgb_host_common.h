// Host-side helpers shared by every translation unit of libfvgb.
#pragma once
#include "fvgb.h"

#ifdef __cplusplus
extern "C" {
#endif
// Record `msg` as this thread's last error and return `st`.
fvgb_status fvgb_fail(fvgb_status st, const char* msg);
// Clear the last error of this thread.
void fvgb_clear_error(void);
#ifdef __cplusplus
}
#endif
