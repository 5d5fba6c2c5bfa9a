// ptrcheck.h -- where an array argument lives, decided from the attributes
// cudaPointerGetAttributes reports for it.
//
// A pointer to device memory of another GPU must not be used in place: a
// kernel on the current device that dereferences it faults unless peer access
// happens to be enabled.  It is rejected on the host instead.  Pure function,
// shared by the library and the host-side emulator (CPU tests).
#pragma once

namespace fg {

enum PtrKind {
  PTR_HOST = 0,         // host memory (pageable or page-locked): staged through a device mirror
  PTR_DEVICE = 1,       // device memory of the current device, or managed memory: used in place
  PTR_OTHER_DEVICE = 2  // device memory of another device: rejected (FLUTAS_EINVAL)
};

// mem_type: cudaPointerAttributes::type as an int (0 unregistered, 1 host,
// 2 device, 3 managed); ptr_device: cudaPointerAttributes::device;
// cur_device: cudaGetDevice().  attr_ok = false when the query itself failed
// (an address the driver does not know: plain host memory).
inline int classify_ptr(bool attr_ok, int mem_type, int ptr_device, int cur_device) {
  if (!attr_ok) return PTR_HOST;
  if (mem_type == 3) return PTR_DEVICE;  // managed: reachable from every device
  if (mem_type == 2) return ptr_device == cur_device ? PTR_DEVICE : PTR_OTHER_DEVICE;
  return PTR_HOST;
}

}  // namespace fg
