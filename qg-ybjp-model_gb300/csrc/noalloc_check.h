// Argument checks of qg_fft_c2r_noalloc that need no GPU: whether a pointer
// described by its cudaPointerAttributes can be handed to a kernel launched
// on the current device, and whether it is aligned for the kernels' vector
// loads.  Plain C++ (the memory type is passed as its integer value) so that
// a host-only test can exercise every branch.
#pragma once
#include <stdint.h>

namespace qgna {

enum PointerVerdict {
  kPointerOk = 0,
  kPointerNotDevice = 1,     // host, pageable or unregistered memory
  kPointerOtherDevice = 2,   // device memory of another GPU
  kPointerMisaligned = 3,
};

// memory_type: cudaPointerAttributes::type (0 unregistered, 1 host,
// 2 device, 3 managed); owner: cudaPointerAttributes::device; current: the
// current device; align: required alignment in bytes (a power of two).
// Managed memory migrates on demand and is accepted on any device.
inline int check_pointer(int memory_type, int owner, int current, const void* p, uintptr_t align) {
  if (memory_type != 2 && memory_type != 3) return kPointerNotDevice;
  if (memory_type == 2 && owner != current) return kPointerOtherDevice;
  if ((reinterpret_cast<uintptr_t>(p) & (align - 1)) != 0) return kPointerMisaligned;
  return kPointerOk;
}

}  // namespace qgna
