// Build harness for the reference's own sDTW kernel (test infrastructure).
//
// Compiles the UNMODIFIED kernel template FullDTW::DTW of
// harisankarsadasivan/DTWax (src/include/DTW.hpp:283 includes
// src/include/DTW.cu:151-572) into a device-only cubin for sm_103a, so the
// reference kernel can be run on a GB300 beside this repository's kernel.
// Only oracle/ref_kernel.py builds this file (nvcc -cubin, with
// -I <reference>/src/include); the cubin goes to oracle/_ref/ and is loaded
// through the CUDA driver API.  Nothing in the product links it.
//
// The reference's configuration header (src/include/common.hpp:28-98) is
// skipped: its include guard tests COMMON_HPP but defines COMON_HPP
// (common.hpp:28-29), so defining COMMON_HPP here keeps it out and the macros
// below take its place.  They carry the reference's values (FP16 half2 or FP32
// arithmetic, 26 cells per lane, 2,048-sample queries in two 1,024-row
// chunks, the derived wave and tile counts) except the reference length,
// which comes from -DHARNESS_REF_LEN so one cubin exists per reference
// geometry (common.hpp:60-67 fixes it at 47*1024 per strand for FP16 and
// 2*47*1024 for FP32).  Build flags follow src/Makefile:8 (-DNO_REF_DEL, and
// -DFP16 for the half2 build); without -DNO_REF_DEL the kernel carries the
// REF_DEL recurrence (DTW.cu:23-29).
//
// <cuda_fp16.h> and <cooperative_groups.h> are included at file scope first:
// DTW.cu includes them again inside namespace FullDTW, where a first inclusion
// would not compile.

#include <cstdint>
#include <cuda_fp16.h>
#include <cooperative_groups.h>

#ifndef HARNESS_REF_LEN
#error "HARNESS_REF_LEN (reference columns: per strand for FP16, both strands for FP32) is required"
#endif

#define COMMON_HPP 1

#ifdef FP16
typedef __half2 value_ht;
#define HALF2FLOAT(a) __half2float(a)
#define FLOAT2HALF(a, b) __floats2half2_rn(a, b)
#define FIND_MIN(a, b) __hmin2(a, b)
#define FMA(a, b, c) __hfma2(a, b, c)
#define ADD(a, b) __hadd2(a, b)
#define SUB(a, b) __hsub2(a, b)
#define SQRT(a) h2sqrt(a)
#define FLOAT2HALF2(a) FLOAT2HALF(a, a)
#define GT(a, b) __hgt(a, b)
#else
typedef float value_ht;
#define FLOAT2HALF(a) a
#define HALF2FLOAT(a) a
#define FIND_MIN(a, b) min(a, b)
#define FIND_MAX(a, b) max(a, b)
#define FMA(a, b, c) __fmaf_ieee_rn(a, b, c)
#define ADD(a, b) (a + b)
#define SUB(a, b) (a - b)
#define SQRT(a) sqrtf(a)
#define FLOAT2HALF2(a) FLOAT2HALF(a)
#define GT(a, b) (a > b)
#endif

#define KMER_LEN 6
#define WARP_SIZE 32
#define LOG_WARP_SIZE 5
#define SEGMENT_SIZE 26
#define QUERY_LEN (512 * 4)
#define PREFIX_LEN (512 * 2)
#define REF_LEN (HARNESS_REF_LEN)
#define BLOCK_NUM (10)
#define STREAM_NUM 1
#define ADAPTER_LEN 1952
#define ONT_FILE_FORMAT "fast5"

#define REF_TILE_SIZE (SEGMENT_SIZE * WARP_SIZE)
#define REF_BATCH (REF_LEN / REF_TILE_SIZE)
#define QUERY_BATCH (QUERY_LEN / PREFIX_LEN)
#define NUM_WAVES (PREFIX_LEN + (REF_TILE_SIZE - 1) / (SEGMENT_SIZE))
#define WARP_SIZE_MINUS_ONE (WARP_SIZE - 1)
#define RESULT_REG (SEGMENT_SIZE - 1)
#define NUM_WAVES_BY_WARP_SIZE ((NUM_WAVES / WARP_SIZE) * WARP_SIZE)
#define REF_BATCH_MINUS_ONE (REF_BATCH - 1)
#define TWICE_WARP_SIZE_MINUS_ONE ((2 * WARP_SIZE) - 1)

#include "DTW.hpp"

static_assert(REF_BATCH >= 2, "the reference kernel needs at least two 832-column tiles");

// The one instantiation the reference's host uses (main.cu:259,
// distances<value_ht, idxt> with idxt = int).
template __global__ void FullDTW::DTW<int, value_ht>(reference_coefficients *, value_ht *, value_ht *, int,
                                                     value_ht, value_ht *);
