// Programmatic dependent launch.  The engine launches its kernels with programmatic
// stream serialization, so a kernel's blocks may be scheduled while its predecessor
// in the stream is still finishing (its launch latency and prologue overlap the
// predecessor's tail).  Every kernel therefore starts by waiting for the predecessor
// grid to complete and its memory to be visible (griddepcontrol.wait; a no-op when
// the launch has no programmatic predecessor, e.g. inside a graph), and then lets its
// own successor be scheduled (griddepcontrol.launch_dependents; the successor still
// waits for this grid's completion before it reads anything).
#pragma once

__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
