// Copy job of the packing pass. Plain types only: the header is also compiled
// at run time by NVRTC together with the entry kernels (hm_entry.cuh).
#pragma once
#ifndef __CUDACC_RTC__
#include <cstdint>
#endif

namespace hm {

// A row-major source slice -> rows of a tile panel.
struct PackJob {
  int64_t src_off;   // element offset in the source array
  int64_t dst_off;   // element offset of (first row, first column) in the panel array
  int32_t src_ld;    // source row stride
  int32_t dst_ld;    // panel row stride
  int32_t ncols;
  int32_t m;         // rows
  int32_t kind;      // 0 dense source, 1 U source, 2 dense generated from the kernel
  int32_t row0;      // generated: first permuted row
  int32_t col0;      // generated: first permuted column
  int32_t pad;
};

}  // namespace hm
