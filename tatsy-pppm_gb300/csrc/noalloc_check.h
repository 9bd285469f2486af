// Pointer rule of pppm_knn_noalloc, kept free of CUDA headers so that a host
// compiler can test it without a GPU. That entry point stages nothing, so
// its kernels read the caller's arrays in place on the current device. A
// pointer qualifies when it is device memory of that same device or managed
// memory (which the driver migrates on access). Host memory, unregistered
// memory and device memory of another GPU (readable only with peer access,
// which the entry point does not set up: the read would be an illegal
// address) are refused.
#ifndef PPPM_NOALLOC_CHECK_H_
#define PPPM_NOALLOC_CHECK_H_

namespace pppm {

// The values of cudaMemoryType (cudaMemoryTypeUnregistered .. Managed).
enum NaMemoryType { kNaUnregistered = 0, kNaHost = 1, kNaDevice = 2, kNaManaged = 3 };

inline bool naPointerUsable(int memoryType, int pointerDevice, int currentDevice) {
    if (memoryType == kNaManaged) return true;
    return memoryType == kNaDevice && pointerDevice == currentDevice;
}

}  // namespace pppm

#endif  // PPPM_NOALLOC_CHECK_H_
