/*
 * ref_cuda_shim.h -- force-included when the reference's cuda/mrg8_cuda.cu is
 * compiled (device code only, into oracle/_ref/) for sm_103a, so that its GPU
 * kernel can be timed beside ours.  TEST INFRASTRUCTURE ONLY.
 *
 * The file uses two calls that CUDA 13 no longer provides: the pre-Volta
 * warp shuffle and the old name of the device synchronisation.  They map to
 * their current forms (full-warp mask; every lane of the warp calls them).
 */
#pragma once
#define __shfl_xor(v, m) __shfl_xor_sync(0xffffffffu, (v), (m))
#define cudaThreadSynchronize cudaDeviceSynchronize
