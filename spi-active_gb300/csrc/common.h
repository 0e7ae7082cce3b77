// common.h -- error reporting and a growable device buffer for the engine's own storage.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstddef>

#include "spi_engine.h"

namespace spi {

int set_error(int code, const char* fmt, ...);
int cuda_error(cudaError_t e, const char* what);

// Engine-owned device allocation that only grows; freed with the engine.
struct DeviceBuf {
  void* p = nullptr;
  size_t cap = 0;
  unsigned generation = 0;   // bumped whenever the allocation moves
  DeviceBuf() = default;
  DeviceBuf(const DeviceBuf&) = delete;
  DeviceBuf& operator=(const DeviceBuf&) = delete;
  ~DeviceBuf() { if (p) cudaFree(p); }
  int reserve(size_t bytes) {
    if (bytes <= cap) return SPI_OK;
    if (p) { cudaFree(p); p = nullptr; cap = 0; }
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return set_error(SPI_ENOMEM, "cudaMalloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
    }
    cap = bytes;
    ++generation;
    return SPI_OK;
  }
  float* f() const { return static_cast<float*>(p); }
  double* d() const { return static_cast<double*>(p); }
};

}  // namespace spi
