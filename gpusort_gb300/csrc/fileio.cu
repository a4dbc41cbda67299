// Per-rank binary files of the reference's test driver
// (src/test/utils.h:610-661, src/test/ifstream.h:38-73,
// src/test/ofstream.h:34-64): file <dir>/<rank><ext> holds a native int64
// element count followed by the raw elements. Device-memory reads and
// writes stream through two pinned staging buffers on the context's stream,
// so the disk and the copies overlap and the data never needs a pageable
// host copy of the whole array.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gpusort_gb300.h"
#include "engine.h"

namespace {

constexpr size_t CHUNK = size_t(32) << 20;  // staging buffer bytes

std::string rank_path(const char* dir, const char* ext, int rank) {
  std::string p(dir);
  p += "/";
  p += std::to_string(rank);
  p += ext ? ext : ".dat";
  return p;
}

// Elements per block of the reference's split (include/common.h:146-155).
uint64_t each_block(uint64_t total, uint64_t p) {
  const uint64_t r = total % p;
  if (r == 0) return total / p;
  const uint64_t tmp = (total + (p - r)) / p;
  return tmp * (p - 1) >= total ? tmp - 1 : tmp;
}

gs_status err(const std::string& m, gs_status st = GS_ERR_INVALID) {
  gs::set_last_global_error(m);
  return st;
}

struct Staging {
  void* buf[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  ~Staging() {
    for (int i = 0; i < 2; ++i) {
      if (ev[i]) {
        cudaEventSynchronize(ev[i]);
        cudaEventDestroy(ev[i]);
      }
      if (buf[i]) cudaFreeHost(buf[i]);
    }
  }
  bool init() {
    for (int i = 0; i < 2; ++i) {
      if (cudaMallocHost(&buf[i], CHUNK) != cudaSuccess) return false;
      if (cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming) != cudaSuccess) return false;
    }
    return true;
  }
};

// Read `bytes` from f into dst (device memory when dev) through staging.
gs_status read_body(FILE* f, uint8_t* dst, uint64_t bytes, bool dev, cudaStream_t st,
                    const std::string& path) {
  if (!dev) {
    if (bytes && std::fread(dst, 1, bytes, f) != bytes) return err("short read from " + path);
    return GS_OK;
  }
  Staging s;
  if (!s.init()) {
    cudaGetLastError();
    return err("pinned staging allocation failed", GS_ERR_OOM);
  }
  uint64_t done = 0;
  for (int k = 0; done < bytes; k ^= 1) {
    const size_t m = size_t(std::min<uint64_t>(CHUNK, bytes - done));
    if (cudaEventSynchronize(s.ev[k]) != cudaSuccess) return err("staging wait", GS_ERR_CUDA);
    if (std::fread(s.buf[k], 1, m, f) != m) return err("short read from " + path);
    if (cudaMemcpyAsync(dst + done, s.buf[k], m, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaEventRecord(s.ev[k], st) != cudaSuccess)
      return err("host to device copy", GS_ERR_CUDA);
    done += m;
  }
  return cudaStreamSynchronize(st) == cudaSuccess ? GS_OK : err("copy", GS_ERR_CUDA);
}

gs_status write_body(FILE* f, const uint8_t* src, uint64_t bytes, bool dev, cudaStream_t st,
                     const std::string& path) {
  if (!dev) {
    if (bytes && std::fwrite(src, 1, bytes, f) != bytes) return err("short write to " + path);
    return GS_OK;
  }
  Staging s;
  if (!s.init()) {
    cudaGetLastError();
    return err("pinned staging allocation failed", GS_ERR_OOM);
  }
  // Copy chunk k+1 while chunk k is written to the file.
  uint64_t issued = 0, written = 0;
  size_t len[2] = {0, 0};
  auto issue = [&](int k) -> bool {
    len[k] = size_t(std::min<uint64_t>(CHUNK, bytes - issued));
    if (len[k] == 0) return true;
    if (cudaMemcpyAsync(s.buf[k], src + issued, len[k], cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaEventRecord(s.ev[k], st) != cudaSuccess)
      return false;
    issued += len[k];
    return true;
  };
  int k = 0;
  if (!issue(0)) return err("device to host copy", GS_ERR_CUDA);
  while (written < bytes) {
    if (cudaEventSynchronize(s.ev[k]) != cudaSuccess) return err("staging wait", GS_ERR_CUDA);
    const size_t m = len[k];
    if (!issue(k ^ 1)) return err("device to host copy", GS_ERR_CUDA);
    if (std::fwrite(s.buf[k], 1, m, f) != m) return err("short write to " + path);
    written += m;
    k ^= 1;
  }
  return GS_OK;
}

}  // namespace

extern "C" {

int64_t gs_file_count(const char* path) {
  if (!path) return -1;
  FILE* f = std::fopen(path, "rb");
  if (!f) return -1;
  int64_t n = -1;
  if (std::fread(&n, sizeof n, 1, f) != 1) n = -1;
  std::fclose(f);
  return n;
}

gs_status gs_file_read(gs_ctx* ctx, const char* path, void* dst, uint64_t capacity,
                       uint32_t elem_bytes, uint32_t flags, uint64_t* n_read) {
  if (!path || elem_bytes == 0) return err("null path or zero element size");
  const bool dev = !(flags & GS_FLAG_HOST);
  if (dev && !ctx) return err("device reads need a context");
  FILE* f = std::fopen(path, "rb");
  if (!f) return err(std::string("cannot open ") + path);
  int64_t n = 0;
  gs_status st = GS_OK;
  if (std::fread(&n, sizeof n, 1, f) != 1 || n < 0) st = err(std::string("no element count in ") + path);
  else if (uint64_t(n) > capacity) st = err(std::string("buffer too small for ") + path, GS_ERR_TOO_LARGE);
  else if (n > 0 && !dst) st = err("null destination");
  if (st == GS_OK)
    st = read_body(f, static_cast<uint8_t*>(dst), uint64_t(n) * elem_bytes, dev,
                   dev ? gs::context_stream(ctx) : nullptr, path);
  std::fclose(f);
  if (st == GS_OK && n_read) *n_read = uint64_t(n);
  return st;
}

gs_status gs_file_write(gs_ctx* ctx, const char* path, const void* src, uint64_t n,
                        uint32_t elem_bytes, uint32_t flags) {
  if (!path || elem_bytes == 0) return err("null path or zero element size");
  if (n > 0 && !src) return err("null source");
  const bool dev = !(flags & GS_FLAG_HOST);
  if (dev && !ctx) return err("device writes need a context");
  cudaStream_t st = dev ? gs::context_stream(ctx) : nullptr;
  if (dev && cudaStreamSynchronize(st) != cudaSuccess) return err("synchronize", GS_ERR_CUDA);
  FILE* f = std::fopen(path, "wb");
  if (!f) return err(std::string("cannot create ") + path);
  const int64_t cnt = int64_t(n);
  gs_status s = std::fwrite(&cnt, sizeof cnt, 1, f) == 1 ? GS_OK : err("short write to " + std::string(path));
  if (s == GS_OK) s = write_body(f, static_cast<const uint8_t*>(src), n * elem_bytes, dev, st, path);
  if (std::fclose(f) != 0 && s == GS_OK) s = err("close failed for " + std::string(path));
  return s;
}

gs_status gs_partitions_read(gs_ctx* ctx, const char* dir, const char* ext, int nparts,
                             void* dst, uint64_t capacity, uint32_t elem_bytes, uint32_t flags,
                             uint64_t* n_total) {
  if (!dir || nparts <= 0) return err("null directory or no partitions");
  uint64_t total = 0;
  for (int r = 0; r < nparts; ++r) {
    const std::string p = rank_path(dir, ext, r);
    const int64_t c = gs_file_count(p.c_str());
    if (c < 0) return err("cannot read the element count of " + p);
    total += uint64_t(c);
  }
  if (total > capacity) return err("buffer too small for the partitions", GS_ERR_TOO_LARGE);
  uint64_t off = 0;
  for (int r = 0; r < nparts; ++r) {
    const std::string p = rank_path(dir, ext, r);
    uint64_t got = 0;
    const gs_status st = gs_file_read(ctx, p.c_str(), static_cast<uint8_t*>(dst) + off * elem_bytes,
                                      capacity - off, elem_bytes, flags, &got);
    if (st != GS_OK) return st;
    off += got;
  }
  if (n_total) *n_total = total;
  return GS_OK;
}

gs_status gs_partitions_write(gs_ctx* ctx, const char* dir, const char* ext, int nparts,
                              const void* src, uint64_t n, uint32_t elem_bytes, uint32_t flags) {
  if (!dir || nparts <= 0) return err("null directory or no partitions");
  const uint64_t each = each_block(n, uint64_t(nparts));
  for (int r = 0; r < nparts; ++r) {
    const uint64_t b = std::min<uint64_t>(each * uint64_t(r), n);
    const uint64_t e = (r == nparts - 1) ? n : std::min<uint64_t>(b + each, n);
    const std::string p = rank_path(dir, ext, r);
    const gs_status st = gs_file_write(ctx, p.c_str(),
                                       static_cast<const uint8_t*>(src) + b * elem_bytes, e - b,
                                       elem_bytes, flags);
    if (st != GS_OK) return st;
  }
  return GS_OK;
}

uint64_t gs_partition_block(uint64_t n, int nparts) {
  return nparts > 0 ? each_block(n, uint64_t(nparts)) : 0;
}

}  // extern "C"
