/*
 * cuda_host_shim.h — lets the reference's CUDA kernel sources compile as
 * host C++ so that they can run on the CPU, one "thread" at a time.
 *
 * TEST INFRASTRUCTURE ONLY (oracle/_ref).  The kernel bodies stay the
 * reference's; this header only supplies what the CUDA compiler would:
 * the built-in thread indices (set by the caller before each call) and
 * sequential stand-ins for the atomics cuNSearch uses.
 */
#pragma once
#include <cuda_runtime.h>

extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;

/* Executed by one host thread in index order, so a plain read-modify-write
 * has the semantics of the device atomic. */
inline int atomicMin(int* a, int v) { int o = *a; if (v < o) *a = v; return o; }
inline int atomicMax(int* a, int v) { int o = *a; if (v > o) *a = v; return o; }
inline unsigned int atomicAdd(unsigned int* a, unsigned int v) { unsigned int o = *a; *a = o + v; return o; }
