/*
 * pt_checked.h — test hooks of the bounds-checked library.
 *
 * libptgpu_checked.so is libptgpu.so's tracer compiled with -DPT_CHECKED:
 * the same entry points (link it instead of libptgpu.so), with every node,
 * triangle, instance, vertex-index and queue index compared with its array's
 * length before use; a bad one makes pt_render fail with PT_ERR_DEVICE,
 * "index out of range", without the read.  The call below exists to prove
 * that on purpose.  It has no counterpart in the reference (whose Vulkan
 * validation layers play this role) and is not part of the rendering API.
 */
#ifndef PT_CHECKED_H_INCLUDED
#define PT_CHECKED_H_INCLUDED

#include "pt_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Overwrites the first child link of the traversed root node of the
 * context's TLAS with `value`; rebuild the acceleration structure to repair
 * it.  Returns PT_ERR_UNSUPPORTED in the normal library (whose kernels do not
 * check) and PT_ERR_STATE when there is no TLAS node (fewer than two
 * instances). */
int pt_debug_poke_tlas_link(pt_ctx* ctx, int value);

#ifdef __cplusplus
}
#endif

#endif /* PT_CHECKED_H_INCLUDED */
