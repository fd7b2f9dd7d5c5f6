/* Declaration-only stand-in for <tskit.h>.
 *
 * Test infrastructure: lets the reference GRGL sources (include/grgl/ts2grg.h,
 * src/grg_helpers.h, src/tskit_util.h) parse when they are compiled here as the
 * CPU oracle.  No tree-sequence code is built; the functions below are linked
 * to stubs that throw (oracle/ref_shim/tsk_stubs.cpp).
 */
#pragma once
#include <stdint.h>
typedef int32_t tsk_id_t;
typedef uint32_t tsk_flags_t;
typedef struct { int unused; } tsk_treeseq_t;
typedef struct { tsk_id_t* parent; tsk_id_t* num_children; } tsk_tree_t;
#define TSK_NULL (-1)
#ifdef __cplusplus
extern "C" {
#endif
int tsk_treeseq_load(tsk_treeseq_t* self, const char* filename, tsk_flags_t options);
int tsk_treeseq_free(tsk_treeseq_t* self);
const char* tsk_strerror(int err);
#ifdef __cplusplus
}
#endif
