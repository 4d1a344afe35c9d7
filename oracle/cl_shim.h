/* ORACLE (test infrastructure only): compiles the reference's generated OpenCL C
 * as C on the host.  OpenCL keywords become C ones, and get_global_id /
 * get_global_size read the work-item coordinates that the OpenMP loop nest of
 * the generated driver sets for each call of the kernel function. */
#ifndef CC_CL_SHIM_H
#define CC_CL_SHIM_H
#include <stdbool.h>
#include <tgmath.h>
#define kernel static inline
#define global
#define restrict __restrict
#ifndef NAN
#define NAN (__builtin_nanf(""))
#endif
static __thread long cl_gid_[3];
static long cl_gsz_[3];
#define get_global_id(d) (cl_gid_[d])
#define get_global_size(d) (cl_gsz_[d])
#endif
