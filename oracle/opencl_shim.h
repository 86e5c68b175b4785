/* Lets an OpenCL C kernel file without barriers or local memory compile as
 * plain C11 on the host (test infrastructure: used only to run the reference's
 * own event kernels on the CPU as a checker).
 *
 * Address-space qualifiers compile away; get_global_id reads the work-item id
 * that the host driver stores in a thread-local array before each call; the
 * OpenCL atomics become GCC __atomic builtins.  The kernel file's compile-time
 * parameters that depend on the dataset (IMAGE_WIDTH, NUM_BINS) are given on
 * the command line as the names of the runtime variables declared here.
 */
#ifndef G2_OPENCL_SHIM_H
#define G2_OPENCL_SHIM_H
#include <stddef.h>
#include <stdint.h>

#define kernel
#define __kernel
#define global
#define __global
#define constant const
typedef unsigned int uint;
typedef unsigned char uchar;
typedef unsigned short ushort;

extern _Thread_local size_t g2r_gid[3];
extern int g2r_image_width;
extern int g2r_num_bins;

static inline size_t get_global_id(int d) { return g2r_gid[d]; }
#define atomic_add(p, v) __atomic_fetch_add((p), (v), __ATOMIC_RELAXED)
#endif
