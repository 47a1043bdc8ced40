// Tensor-core (tcgen05) vertex contraction for batched evaluation.
#include "evaluate.cuh"

namespace tnfa {

bool tc_vertex_eligible(int, const int*, int) { return false; }
void tc_prepare_net(tnfa_ctx*, const tnfa_net*) {}
int tc_tile_rows() { return 128; }
void tc_contract_vertex(tnfa_ctx*, const tnfa_net*, int, const VertexJob<float>&, int) {
  fail(TNFA_ERR_UNSUPPORTED, "tensor-core evaluation not built");
}

}  // namespace tnfa
