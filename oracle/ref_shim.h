/*
 * ref_shim.h -- lets the reference's OpenCL C kernel sources compile as host
 * C++ so that they can serve as the parity pin for the oracle restatement.
 * TEST INFRASTRUCTURE ONLY (see oracle/build_ref.sh).
 *
 * The kernels use only scalar FP64 C, private variables and the work-item id,
 * so defining the address-space qualifiers away and supplying a per-thread
 * work-item id is enough.  barrier() is a no-op: every work-item runs to
 * completion before the next one starts, and the kernels never communicate
 * through local memory.  The debug printf at Gid==1 is silenced.
 */
#ifndef CFD_REF_SHIM_H
#define CFD_REF_SHIM_H
#include <cmath>
#include <cstdio>

#define __kernel
#define __global
#define __private
#define __constant const
#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2
typedef unsigned int uint;

extern thread_local unsigned shim_gid;
static inline unsigned get_global_id(int) { return shim_gid; }
static inline unsigned get_local_id(int) { return 0u; }
static inline void barrier(int) {}
#define printf(...) ((void)0)

using std::sqrt;
using std::pow;
using std::fabs;
using std::cbrt;
#endif
