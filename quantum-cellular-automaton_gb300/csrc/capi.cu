// Error capture and library-level entry points of the C ABI.
#include <atomic>
#include <cstdarg>

#include "common.cuh"

namespace qca {

namespace {
thread_local char g_error[1024] = "";
std::atomic<long long> g_launches{0};
}

void count_launches(int k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

long long launches_so_far() { return g_launches.load(std::memory_order_relaxed); }

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_error, sizeof(g_error), fmt, ap);
  va_end(ap);
}

const char* last_error() { return g_error; }

}  // namespace qca

extern "C" {

const char* qca_last_error(void) { return qca::last_error(); }

int qca_version(void) { return 100; }

int qca_device_count(int* count) {
  if (!count) {
    qca::set_error("qca_device_count: NULL argument");
    return QCA_ERR_INVALID;
  }
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    n = 0;
  }
  *count = n;
  return QCA_OK;
}

}  // extern "C"
