// Error status and launch accounting.
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>

#include <atomic>

#include "eg_internal.h"

namespace eg {

static thread_local int t_code = 0;
static thread_local char t_msg[512] = {0};
static std::atomic<int> g_abort{-1};
static std::atomic<int64_t> g_launches{0};

static bool abort_mode() {
  int v = g_abort.load();
  if (v < 0) {
    const char *e = getenv("EINSPLINE_GB300_ABORT");
    v = (e && e[0] == '0') ? 0 : 1;
    g_abort.store(v);
  }
  return v != 0;
}

int fail(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(t_msg, sizeof(t_msg), fmt, ap);
  va_end(ap);
  t_code = code;
  if (abort_mode()) {
    fprintf(stderr, "einspline_gb300 error %d: %s\n", code, t_msg);
    abort();
  }
  return code;
}

void clear() {
  t_code = 0;
  t_msg[0] = 0;
}

int cuda_check(cudaError_t e, const char *what) {
  cudaGetLastError();
  return fail(EINSPLINE_GB300_ECUDA, "CUDA error in %s: %s", what, cudaGetErrorString(e));
}

void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

}  // namespace eg

extern "C" {

int einspline_gb300_last_error(void) { return eg::t_code; }
const char *einspline_gb300_last_error_message(void) { return eg::t_msg; }
void einspline_gb300_clear_error(void) { eg::clear(); }
void einspline_gb300_set_abort_on_error(int enable) { eg::g_abort.store(enable ? 1 : 0); }
int64_t einspline_gb300_launch_count(void) { return eg::g_launches.load(); }

}
