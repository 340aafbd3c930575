// Raster I/O between files and device memory: the GPU-side analogue of the
// callers' GDAL step before the D8 path.  A file is moved in chunks through
// two pinned host buffers: while one chunk is copied to (or from) the device
// on the caller's stream, the next one is read from (or the previous one
// written to) the file, so disk throughput and PCIe / NVLink-C2C copies
// overlap.  The pinned buffers are allocated once per device and reused.
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <mutex>

#include "tt_internal.cuh"

namespace tt {
namespace {

constexpr size_t kIoChunk = size_t(16) << 20;  // 16 MiB per pinned buffer
constexpr int kIoDevices = 64;

struct IoBuffers {
  char *buf[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
};
IoBuffers g_io[kIoDevices];
std::mutex g_io_mu[kIoDevices];

tt_cuda_status io_buffers(int dev, IoBuffers **out) {
  if (dev < 0 || dev >= kIoDevices) return TT_CUDA_ERR_INVALID_ARGUMENT;
  IoBuffers &b = g_io[dev];
  for (int k = 0; k < 2; k++) {
    if (!b.buf[k] && cudaHostAlloc((void **)&b.buf[k], kIoChunk, cudaHostAllocDefault) != cudaSuccess) {
      cudaGetLastError();
      b.buf[k] = nullptr;
      return TT_CUDA_ERR_ALLOC;
    }
    if (!b.done[k] && cudaEventCreateWithFlags(&b.done[k], cudaEventDisableTiming) != cudaSuccess) {
      cudaGetLastError();
      b.done[k] = nullptr;
      return TT_CUDA_ERR_CUDA;
    }
  }
  *out = &b;
  return TT_CUDA_SUCCESS;
}

// Reads exactly `len` bytes at `off` (retrying short reads).
bool read_full(int fd, char *p, size_t len, int64_t off) {
  while (len) {
    const ssize_t r = pread(fd, p, len, (off_t)off);
    if (r <= 0) return false;
    p += r;
    len -= (size_t)r;
    off += r;
  }
  return true;
}

bool write_full(int fd, const char *p, size_t len, int64_t off) {
  while (len) {
    const ssize_t r = pwrite(fd, p, len, (off_t)off);
    if (r <= 0) return false;
    p += r;
    len -= (size_t)r;
    off += r;
  }
  return true;
}

tt_cuda_status read_file(char *dst, int fd, int64_t offset, int64_t bytes, IoBuffers &b,
                         cudaStream_t st) {
  int64_t done = 0;
  for (int k = 0; done < bytes; k ^= 1) {
    const size_t len = (size_t)std::min<int64_t>((int64_t)kIoChunk, bytes - done);
    // the previous copy out of this buffer must have finished
    TT_CHECK(cudaEventSynchronize(b.done[k]));
    if (!read_full(fd, b.buf[k], len, offset + done)) return TT_CUDA_ERR_IO;
    TT_CHECK(cudaMemcpyAsync(dst + done, b.buf[k], len, cudaMemcpyHostToDevice, st));
    TT_CHECK(cudaEventRecord(b.done[k], st));
    done += (int64_t)len;
  }
  TT_CHECK(cudaStreamSynchronize(st));
  return TT_CUDA_SUCCESS;
}

// Chunk c goes through buffer c % 2: the copy of chunk c + 1 is issued
// before chunk c is written, and a buffer is refilled only after its
// previous chunk has been written (writes are synchronous here).
tt_cuda_status write_file(int fd, int64_t offset, const char *src, int64_t bytes, IoBuffers &b,
                          cudaStream_t st) {
  const int64_t nchunks = (bytes + (int64_t)kIoChunk - 1) / (int64_t)kIoChunk;
  auto len_of = [&](int64_t c) {
    return (size_t)std::min<int64_t>((int64_t)kIoChunk, bytes - c * (int64_t)kIoChunk);
  };
  if (nchunks > 0) {
    TT_CHECK(cudaMemcpyAsync(b.buf[0], src, len_of(0), cudaMemcpyDeviceToHost, st));
    TT_CHECK(cudaEventRecord(b.done[0], st));
  }
  for (int64_t c = 0; c < nchunks; c++) {
    const int k = (int)(c & 1);
    if (c + 1 < nchunks) {
      TT_CHECK(cudaMemcpyAsync(b.buf[k ^ 1], src + (c + 1) * (int64_t)kIoChunk, len_of(c + 1),
                               cudaMemcpyDeviceToHost, st));
      TT_CHECK(cudaEventRecord(b.done[k ^ 1], st));
    }
    TT_CHECK(cudaEventSynchronize(b.done[k]));
    if (!write_full(fd, b.buf[k], len_of(c), offset + c * (int64_t)kIoChunk)) return TT_CUDA_ERR_IO;
  }
  return TT_CUDA_SUCCESS;
}

bool have_gpu() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return n > 0;
}

}  // namespace
}  // namespace tt

extern "C" tt_cuda_status tt_cuda_read_file_dev(void *dst, const char *path, int64_t offset,
                                                int64_t bytes, void *stream) {
  using namespace tt;
  tt_cuda_status s = TT_CUDA_SUCCESS;
  if (!dst || !path || offset < 0 || bytes < 0) {
    s = TT_CUDA_ERR_INVALID_ARGUMENT;
  } else if (!have_gpu()) {
    s = TT_CUDA_ERR_NO_DEVICE;
  } else {
    const int fd = open(path, O_RDONLY);
    if (fd < 0) {
      s = TT_CUDA_ERR_IO;
    } else {
      int dev = 0;
      cudaGetDevice(&dev);
      IoBuffers *b = nullptr;
      std::lock_guard<std::mutex> lock(g_io_mu[dev < kIoDevices && dev >= 0 ? dev : 0]);
      s = io_buffers(dev, &b);
      if (s == TT_CUDA_SUCCESS) s = read_file((char *)dst, fd, offset, bytes, *b, (cudaStream_t)stream);
      close(fd);
    }
  }
  if (s == TT_CUDA_ERR_CUDA) cudaGetLastError();
  set_status(s);
  return s;
}

extern "C" tt_cuda_status tt_cuda_write_file_dev(const char *path, int64_t offset,
                                                 const void *src, int64_t bytes, void *stream) {
  using namespace tt;
  tt_cuda_status s = TT_CUDA_SUCCESS;
  if (!src || !path || offset < 0 || bytes < 0) {
    s = TT_CUDA_ERR_INVALID_ARGUMENT;
  } else if (!have_gpu()) {
    s = TT_CUDA_ERR_NO_DEVICE;
  } else {
    const int fd = open(path, O_WRONLY | O_CREAT, 0644);
    if (fd < 0) {
      s = TT_CUDA_ERR_IO;
    } else {
      int dev = 0;
      cudaGetDevice(&dev);
      IoBuffers *b = nullptr;
      std::lock_guard<std::mutex> lock(g_io_mu[dev < kIoDevices && dev >= 0 ? dev : 0]);
      s = io_buffers(dev, &b);
      if (s == TT_CUDA_SUCCESS)
        s = write_file(fd, offset, (const char *)src, bytes, *b, (cudaStream_t)stream);
      if (close(fd) != 0 && s == TT_CUDA_SUCCESS) s = TT_CUDA_ERR_IO;
    }
  }
  if (s == TT_CUDA_ERR_CUDA) cudaGetLastError();
  set_status(s);
  return s;
}
