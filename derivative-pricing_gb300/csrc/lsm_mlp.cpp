// lsm_mlp.cpp -- placeholder until the learned regression lands.
#include "lsm_mlp.hpp"

namespace mcdg {

int lsm_mlp_batch(Ctx& ctx, const mcd_lsm_contract*, size_t, int, mcd_lsm_result*) {
    return ctx.fail(MCD_ERR_UNSUPPORTED, "learned LSM regression is not built yet");
}

}  // namespace mcdg
