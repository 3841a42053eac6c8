// Argument checks of the entry points that take caller-owned device buffers
// (host code, no CUDA types, so that a CPU test can run every branch).
#pragma once

namespace rflu {

// What cudaPointerGetAttributes reports about a caller's pointer.
enum class ArgMem { Unknown, Host, Device, Managed };

// The problem with handing a caller's pointer to a kernel of a context that
// lives on ctxDevice while currentDevice is current, or nullptr when there is
// none.  Device memory must sit on the context's device (a kernel would read
// another GPU's memory as a peer access, or fault without peer access);
// managed memory migrates to whichever GPU touches it; host memory and
// pointers CUDA does not know are refused.
inline const char *deviceArgProblem(ArgMem kind, int ptrDevice, int ctxDevice, int currentDevice) {
  if (currentDevice != ctxDevice) return "the current device is not the device the context was created on";
  if (kind == ArgMem::Managed) return nullptr;
  if (kind != ArgMem::Device) return "the buffers must be device (or managed) memory";
  if (ptrDevice != ctxDevice) return "a buffer lives on another device than the context";
  return nullptr;
}

}  // namespace rflu
