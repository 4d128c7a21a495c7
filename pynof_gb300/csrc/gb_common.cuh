// Shared status handling for the libpynof_gb300 C ABI.
//
// Every exported entry point returns an int status (GB_OK == 0) and records a
// human-readable message retrievable with gb_last_error() (thread-local).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <string>

#include "../../include/pynof_gb300.h"

namespace gb {

void set_error(int code, const char* fmt, ...);
void clear_error();

// Launch profiler hooks (profile.cu): prof_begin returns -1 when disabled.
int prof_begin(const char* name, cudaStream_t s);
void prof_end(int idx, cudaStream_t s);

// Id of the calling thread's current CUDA context (cuCtxGetId; unique for the
// life of the process, so a context re-created after cudaDeviceReset gets a
// new one), 0 when there is none.
unsigned long long current_context_id();

// Device address of the tensor-core status word (GB_OK, or the first
// GB_ERR_TIMEOUT / GB_ERR_NONFINITE a kernel recorded) on the current device;
// nullptr if it cannot be looked up.  Looked up once per device context.
int* device_status_word();

// Round up to a multiple of 256 bytes (every workspace carve is 256-aligned).
inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Bump allocator over a caller-provided workspace.
struct Carve {
  char* base;
  size_t cap;
  size_t used = 0;
  Carve(void* p, size_t c) : base(static_cast<char*>(p)), cap(c) {}
  template <class T>
  T* take(size_t count) {
    size_t bytes = align256(count * sizeof(T));
    if (used + bytes > cap) return nullptr;
    T* r = reinterpret_cast<T*>(base + used);
    used += bytes;
    return r;
  }
};

// A Carve that only counts: run a layout function over it to size a workspace.
struct SizeCarve {
  size_t used = 0;
  template <class T>
  T* take(size_t count) {
    used += align256(count * sizeof(T));
    return nullptr;
  }
};

// Size bookkeeping with the same rounding as Carve.
struct Sizer {
  size_t used = 0;
  template <class T>
  void add(size_t count) { used += align256(count * sizeof(T)); }
};

inline int cuda_status(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return GB_OK;
  set_error(GB_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
  return GB_ERR_CUDA;
}

}  // namespace gb

#define GB_CHECK_LAUNCH(where)                                                   \
  do {                                                                           \
    cudaError_t _e = cudaGetLastError();                                         \
    if (_e != cudaSuccess) return gb::cuda_status(_e, where);                    \
  } while (0)

// Launch a kernel under the optional profiler and check the launch.
#define GB_LAUNCH(name, stream, ...)                                             \
  do {                                                                           \
    const int _pi = gb::prof_begin(name, stream);                                \
    __VA_ARGS__;                                                                 \
    gb::prof_end(_pi, stream);                                                   \
    GB_CHECK_LAUNCH(name);                                                       \
  } while (0)

#define GB_TRY(expr)                                                             \
  do {                                                                           \
    int _s = (expr);                                                             \
    if (_s != GB_OK) return _s;                                                  \
  } while (0)

#define GB_REQUIRE(cond, code, ...)                                              \
  do {                                                                           \
    if (!(cond)) {                                                               \
      gb::set_error(code, __VA_ARGS__);                                          \
      return code;                                                               \
    }                                                                            \
  } while (0)
