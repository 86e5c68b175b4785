/* Lets an OpenCL C kernel file that uses work-group barriers and local
 * memory compile as plain C11 on the host -- test infrastructure only: it
 * runs the reference's own dense and CSR kernels on the CPU as checkers.
 *
 * The host driver (ref_wg_driver.c) runs ONE work-group at a time, its
 * work-items as POSIX threads.  So:
 *   - `local` arrays become function-scope statics, shared by the threads of
 *     the running group (groups never overlap, and every group's kernel code
 *     initialises them itself, as OpenCL requires);
 *   - barrier() waits for every thread of the group that is still inside the
 *     kernel body; a thread that has returned counts as arrived.  This is how
 *     the reference's kernels behave on the GPUs they were written for, where
 *     some barriers sit inside `if (tid < 32) { ... }` blocks that only one
 *     warp enters (correlator.cl:85-108); a plain barrier over all the group's
 *     threads would wait forever there.  The barrier (a mutex and a condition
 *     variable) also orders the threads' memory accesses;
 *   - get_local_id / get_group_id / get_global_id read thread-local ids set by
 *     the driver before each call;
 *   - the OpenCL atomics become GCC __atomic builtins.
 * OpenCL's `char` is signed: build with -fsigned-char so that the dense
 * kernel reads its frames as the reference does on every host.
 * The kernel file's compile-time parameters (IMAGE_WIDTH, NUM_BINS, ...) are
 * given on the gcc command line exactly as the reference passes them to the
 * OpenCL compiler.
 */
#ifndef G2_OPENCL_WG_SHIM_H
#define G2_OPENCL_WG_SHIM_H
#include <pthread.h>
#include <stddef.h>
#include <stdint.h>

#define kernel
#define __kernel
#define global
#define __global
#define local static
#define __local static
#define constant const
typedef unsigned int uint;
typedef unsigned char uchar;
typedef unsigned short ushort;

extern _Thread_local size_t g2w_lid[3];
extern _Thread_local size_t g2w_grp[3];
extern size_t g2w_lsize[3];
void g2w_barrier(void);

static inline size_t get_local_id(int d) { return g2w_lid[d]; }
static inline size_t get_group_id(int d) { return g2w_grp[d]; }
static inline size_t get_local_size(int d) { return g2w_lsize[d]; }
static inline size_t get_global_id(int d) { return g2w_grp[d] * g2w_lsize[d] + g2w_lid[d]; }

#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2
static inline void barrier(int flags) {
  (void)flags;
  g2w_barrier();
}
#define atomic_add(p, v) __atomic_fetch_add((p), (v), __ATOMIC_SEQ_CST)
#endif
