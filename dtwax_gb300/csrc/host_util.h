// Host-side helpers of libdtwx: device buffers, FASTA and k-mer model parsing.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace dtwx {

// Device buffer that grows on demand (contents are not preserved on growth).
struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = bytes < 256 ? 256 : bytes;
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <typename T> T *as() const { return static_cast<T *>(p); }
};

// Pinned host buffer that grows on demand.
struct HostBuf {
  void *p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap && p) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    size_t want = bytes < 4096 ? 4096 : bytes + bytes / 4;
    cudaError_t e = cudaMallocHost(&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
  }
  template <typename T> T *as() const { return static_cast<T *>(p); }
};

// Single-record FASTA reader with the rules of load_reference::ref_loader
// (src/include/load_reference.hpp:164-212): a line starting with '>' or an
// empty line ends the current record; a sequence line containing a space
// invalidates the current record; the last valid record wins.  Carriage
// returns are stripped (Windows line ends).  Returns false with a message when
// no record survives.
bool parse_fasta(const std::string &text, std::string &seq, std::string &name, std::string &err);

// k-mer model text "KMER mean stdev" per line (read_kmer_model,
// src/include/load_reference.hpp:131-161).  Fills table[4096] by 2-bit code
// (A<C<G<T, first base most significant).  Every 6-mer must be present.
bool parse_kmer_model(const std::string &text, std::vector<double> &table, std::string &err);

bool read_file(const std::string &path, std::string &out);

}  // namespace dtwx
