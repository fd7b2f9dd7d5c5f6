// Link stubs for the tree-sequence entry points the reference sources reference.
// Test infrastructure only: tskit is not available, so every call throws.
#include <stdexcept>
#include "tskit.h"
#include "grgl/ts2grg.h"

extern "C" int tsk_treeseq_load(tsk_treeseq_t*, const char*, tsk_flags_t) {
    throw std::runtime_error("tskit is not available in this oracle build");
}
extern "C" int tsk_treeseq_free(tsk_treeseq_t*) { return 0; }
extern "C" const char* tsk_strerror(int) { return "tskit is not available in this oracle build"; }

namespace grgl {
MutableGRGPtr convertTreeSeqToGRG(const tsk_treeseq_t*, bool, bool, bool, bool, std::pair<size_t, size_t>) {
    throw std::runtime_error("tskit is not available in this oracle build");
}
} // namespace grgl
