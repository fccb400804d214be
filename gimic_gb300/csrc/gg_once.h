// One-time set-up per CUDA device, safe under concurrent first calls.
//
// Kernel attributes (cudaFuncSetAttribute) and device properties apply to
// the device that is current when they are set or read, so the launchers
// keep one flag per device instead of one per process: every device gets
// its own set-up on its first launch, and threads that make their first
// calls at the same time wait for the one that runs it.
#pragma once
#include <cuda_runtime.h>

#include <mutex>

namespace gg {

constexpr int kMaxDevices = 64;

struct PerDevice {
  std::once_flag flag[kMaxDevices];
  cudaError_t rc[kMaxDevices] = {};
  int value[kMaxDevices] = {};
};

// Runs f(device, &value) once for the current device and returns its
// status (the same status on every later call); *value_out receives the
// int that f stored for this device.
template <typename F>
cudaError_t once_per_device(PerDevice& pd, int* value_out, F f) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::call_once(pd.flag[dev], [&] { pd.rc[dev] = f(dev, &pd.value[dev]); });
  if (value_out) *value_out = pd.value[dev];
  return pd.rc[dev];
}

}  // namespace gg
