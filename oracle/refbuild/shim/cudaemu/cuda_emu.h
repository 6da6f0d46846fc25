/* Runs CUDA C++ kernels of the reference on the CPU, one thread after the
 * other in launch order, so that the reference's own kernel source produces
 * golden data without a GPU (oracle build recipe only).  The recipe rewrites
 * every `kern<<<grid, block>>>(args);` into ORACLE_EMU_LAUNCH((grid, block),
 * kern(args)); atomics are plain read-modify-writes, which is one legal
 * interleaving of the reference's threads. */
#ifndef ORACLE_EMU_CUDA_EMU_H
#define ORACLE_EMU_CUDA_EMU_H
#include <cfloat>
#include <cmath>
#include <cstdint>
#include "cuda_runtime.h"

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline

inline thread_local uint3 threadIdx, blockIdx;
inline thread_local dim3 blockDim, gridDim;

static inline int __clz(int x) { return x ? __builtin_clz((unsigned)x) : 32; }
static inline unsigned atomicAdd(unsigned *a, unsigned v) { unsigned o = *a; *a = o + v; return o; }

struct oracle_emu_cfg {
	dim3 g, b;
	oracle_emu_cfg(dim3 gg, dim3 bb) : g(gg), b(bb) {}
};

#define ORACLE_EMU_LAUNCH(cfg, call)                                                   \
	do {                                                                               \
		oracle_emu_cfg _oc cfg;                                                        \
		gridDim = _oc.g; blockDim = _oc.b;                                             \
		for (unsigned _bz = 0; _bz < _oc.g.z; ++_bz)                                   \
		for (unsigned _by = 0; _by < _oc.g.y; ++_by)                                   \
		for (unsigned _bx = 0; _bx < _oc.g.x; ++_bx)                                   \
		for (unsigned _tz = 0; _tz < _oc.b.z; ++_tz)                                   \
		for (unsigned _ty = 0; _ty < _oc.b.y; ++_ty)                                   \
		for (unsigned _tx = 0; _tx < _oc.b.x; ++_tx) {                                 \
			blockIdx.x = _bx; blockIdx.y = _by; blockIdx.z = _bz;                      \
			threadIdx.x = _tx; threadIdx.y = _ty; threadIdx.z = _tz;                   \
			call;                                                                      \
		}                                                                              \
	} while (0)
#endif
