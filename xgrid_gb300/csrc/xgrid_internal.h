// Runtime hooks used only by generated kernel modules (not part of the public C ABI).
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

/* While `on` is nonzero on the calling thread, the runtime refuses to allocate
 * device memory for boundary-mask tables and reports an error instead.  The
 * no-alloc entry points of generated modules set it around their call. */
void xg_internal_noalloc_scope(int on);

#ifdef __cplusplus
}
#endif
