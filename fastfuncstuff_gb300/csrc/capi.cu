// Library-wide C entry points: version, status strings and the per-thread
// error message behind ffs_last_error().
#include <stdarg.h>

#include "common.cuh"

namespace ffsk {

static thread_local char g_err[1024] = {0};

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

void clear_error() { g_err[0] = 0; }

int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return FFS_ERR_CUDA;
  }
  return FFS_OK;
}

}  // namespace ffsk

extern "C" int ffs_version(void) { return (1 << 16) | 0; }

extern "C" const char* ffs_status_string(int status) {
  switch (status) {
    case FFS_OK: return "ok";
    case FFS_ERR_INVALID: return "invalid argument";
    case FFS_ERR_CUDA: return "CUDA error";
    case FFS_ERR_UNSUPPORTED: return "unsupported shape";
    case FFS_ERR_WORKSPACE: return "workspace too small";
    case FFS_ERR_TIMEOUT: return "device-side wait timed out";
    default: return "unknown status";
  }
}

extern "C" const char* ffs_last_error(void) { return ffsk::g_err; }

extern "C" int ffs_device_view(const void* host_ptr, const void** dev_ptr) {
  ffsk::clear_error();
  FFS_REQUIRE(host_ptr && dev_ptr, "ffs_device_view: null argument");
  cudaPointerAttributes at;
  const cudaError_t e = cudaPointerGetAttributes(&at, host_ptr);
  if (e != cudaSuccess) {
    cudaGetLastError();  // the failed query leaves no error for later launch checks
    ffsk::set_error("ffs_device_view: cudaPointerGetAttributes: %s", cudaGetErrorString(e));
    return FFS_ERR_INVALID;
  }
  if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) {
    *dev_ptr = at.devicePointer ? at.devicePointer : host_ptr;
    return FFS_OK;
  }
  FFS_REQUIRE(at.type == cudaMemoryTypeHost && at.devicePointer,
              "ffs_device_view: %p is not pinned host memory mapped into the device's address space", host_ptr);
  *dev_ptr = at.devicePointer;
  return FFS_OK;
}
