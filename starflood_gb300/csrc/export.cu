// export.cu -- the tree in the reference's node_t numbering (filled in below).
#include "internal.cuh"
#include "tree.cuh"

int sf_tree_export(sfgpu_sim* s, uint32_t*, uint32_t*, uint32_t*, float*, float*) {
    (void)s;
    sf_set_error("tree export is not available in this build");
    return SFGPU_FAILURE;
}
