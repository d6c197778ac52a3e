// Build input straight from a raw row-major float32 file: the format of the
// reference's loadbinData (src/Utilities.cpp:142-214), which mmaps the file
// and copies every row into an in-memory matrix. Here the mapped pages are
// copied chunk by chunk into two pinned buffers and sent to the device while
// the next chunk is copied, so the rows never have to fit in host memory at
// once; the device zero-pads them to the row stride.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include "core.h"

using namespace ceos_host;

namespace {

struct Mapping {
  void* p = MAP_FAILED;
  size_t bytes = 0;
  ~Mapping() {
    if (p != MAP_FAILED) munmap(p, bytes);
  }
};

struct Pinned2 {
  void* b[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  ~Pinned2() {
    for (int i = 0; i < 2; ++i) {
      if (ev[i]) {
        cudaEventSynchronize(ev[i]);
        cudaEventDestroy(ev[i]);
      }
      if (b[i]) cudaFreeHost(b[i]);
    }
  }
};

}  // namespace

int Core::upload_rows_from_file(const char* path, long n, float* dst) {
  if (n <= 0) return CEOS_OK;
  const int fd = open(path, O_RDONLY);
  if (fd < 0) return fail(CEOS_ERR_ARG, "cannot open %s", path);
  struct stat sb;
  if (fstat(fd, &sb) != 0) {
    close(fd);
    return fail(CEOS_ERR_ARG, "cannot stat %s", path);
  }
  const size_t row_bytes = (size_t)n_features * 4;
  const size_t total_rows = (size_t)sb.st_size / row_bytes;
  if ((size_t)n > total_rows) {  // src/Utilities.cpp:171-175
    close(fd);
    return fail(CEOS_ERR_ARG, "numPoints (%ld) exceeds the number of rows in the file (%zu)", n, total_rows);
  }
  Mapping map;
  map.bytes = (size_t)n * row_bytes;
  map.p = mmap(nullptr, map.bytes, PROT_READ, MAP_PRIVATE, fd, 0);
  close(fd);
  if (map.p == MAP_FAILED) return fail(CEOS_ERR_ARG, "cannot map %s", path);
  madvise(map.p, map.bytes, MADV_SEQUENTIAL);

  const size_t chunk_rows = std::max<size_t>(1, ((size_t)32 << 20) / row_bytes);
  const size_t chunk_bytes = chunk_rows * row_bytes;
  Pinned2 pin;
  for (int i = 0; i < 2; ++i) {
    CUDA_TRY(cudaHostAlloc(&pin.b[i], chunk_bytes, cudaHostAllocDefault));
    CUDA_TRY(cudaEventCreateWithFlags(&pin.ev[i], cudaEventDisableTiming));
  }
  if (ldx != n_features) CUDA_TRY(wStage.ensure(2 * chunk_bytes));
  const unsigned char* src = static_cast<const unsigned char*>(map.p);
  int k = 0;
  for (size_t r0 = 0; r0 < (size_t)n; r0 += chunk_rows, k ^= 1) {
    const size_t nr = std::min(chunk_rows, (size_t)n - r0);
    CUDA_TRY(cudaEventSynchronize(pin.ev[k]));  // the copy that last used this buffer is done
    std::memcpy(pin.b[k], src + r0 * row_bytes, nr * row_bytes);
    if (ldx == n_features) {
      CUDA_TRY(cudaMemcpyAsync(dst + r0 * ldx, pin.b[k], nr * row_bytes, cudaMemcpyHostToDevice, stream));
    } else {
      float* stage = wStage.as<float>() + (size_t)k * chunk_rows * n_features;
      CUDA_TRY(cudaMemcpyAsync(stage, pin.b[k], nr * row_bytes, cudaMemcpyHostToDevice, stream));
      CUDA_TRY(launch_pad_rows(stage, (long)nr, n_features, dst + r0 * ldx, ldx, stream));
    }
    CUDA_TRY(cudaEventRecord(pin.ev[k], stream));
  }
  CUDA_TRY(cudaStreamSynchronize(stream));
  return CEOS_OK;
}
