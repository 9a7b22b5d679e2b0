// Internal: set the calling thread's last-error message (read by
// weno_last_error).  Not exported from the library.
#pragma once

namespace weno {
__attribute__((visibility("hidden"))) int set_last_error(int code, const char* msg);
}
