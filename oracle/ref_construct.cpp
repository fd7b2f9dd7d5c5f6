// Test infrastructure: drives the reference GRGL constructor to turn a VCF/IGD into a
// .grg file, with the settings `grg construct` passes to its per-part `grgl` call
// (pygrgl/clicmd/construct.py:219-257 -> src/grgl.cpp:297-369): --trees optimal
// (treeCount 0, no FASTER flags), --lf-no-tree 10, --reduce 5 (min drop 1000,
// fraction 0.8), missing data emitted unless "--ignore-missing" is given, FORCE set.
//
// usage: ref_construct <input.vcf[.gz]|.igd> <output.grg> [--ignore-missing]
#include "fast_build.h"
#include "grgl/grg.h"
#include "grgl/serialize.h"
#include "grgl/transform.h"

#include <cstring>
#include <iostream>
#include <map>

int main(int argc, char** argv) {
    if (argc < 3) {
        std::cerr << "usage: ref_construct <input> <output.grg> [--ignore-missing]\n";
        return 2;
    }
    const std::string input = argv[1];
    const std::string output = argv[2];
    const bool ignoreMissing = (argc > 3 && 0 == strcmp(argv[3], "--ignore-missing"));
    grgl::MutationIteratorFlags itFlags = grgl::MIT_FLAG_FORCE;
    if (!ignoreMissing) {
        itFlags = (grgl::MutationIteratorFlags)(itFlags | grgl::MIT_FLAG_EMIT_MISSING_DATA);
    }
    grgl::FloatRange range;
    std::map<std::string, std::string> noPops;
    grgl::MutableGRGPtr g = grgl::fastGRGFromSamples(
        output, input, range, grgl::GBF_EMPTY, itFlags, /*treeCount=*/0, /*noTreeBelow=*/10.0, noPops);
    grgl::reduceGRGUntil(g, 5, 1000, 0.8);
    grgl::saveGRG(g, output, true);
    grgl::GRGPtr im = grgl::loadImmutableGRG(output, false);
    std::cout << "{\"samples\": " << im->numSamples() << ", \"mutations\": " << im->numMutations()
              << ", \"nodes\": " << im->numNodes() << ", \"edges\": " << im->numEdges() << "}\n";
    return 0;
}
