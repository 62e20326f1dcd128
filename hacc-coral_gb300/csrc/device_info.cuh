// device_info.cuh -- launch sizing from the device's own attributes.
#pragma once

#include <atomic>

#include <cuda_runtime.h>

namespace hsr {

// Streaming multiprocessors of the current device, looked up once per device
// (the grid caps of the grid-stride kernels are multiples of it).  1 when the
// query fails, so a cap never reaches 0.
inline int sm_count() {
  constexpr int kDevices = 64;
  static std::atomic<int> cache[kDevices];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (dev >= 0 && dev < kDevices) {
    const int c = cache[dev].load(std::memory_order_relaxed);
    if (c > 0) return c;
  }
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
    sms = 1;
  if (dev >= 0 && dev < kDevices) cache[dev].store(sms, std::memory_order_relaxed);
  return sms;
}

}  // namespace hsr
