// Entry points whose device implementation is not in this build yet.  Each
// returns TNFA_ERR_UNSUPPORTED with a message instead of computing on the host.
#include "common.cuh"

#define TNFA_PENDING(name)                                                    \
  TNFA_API_BEGIN(ctx);                                                        \
  require_ctx(ctx);                                                           \
  tnfa::fail(TNFA_ERR_UNSUPPORTED, name " is not implemented in this build"); \
  TNFA_API_END

using namespace tnfa;

extern "C" {

int tnfa_partial_integrate(tnfa_ctx* ctx, const tnfa_net*, int32_t, const int32_t*, int,
                           tnfa_net**) {
  TNFA_PENDING("tnfa_partial_integrate")
}

}  // extern "C"
