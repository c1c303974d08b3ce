// mlmc.cu -- multilevel Monte Carlo controller (placeholder).
#include "engine.h"

extern "C" myql_status myql_mlmc_price(myql_ctx *, const myql_mc_job *, const myql_mlmc_config *,
                                       myql_mlmc_result *) {
  return myql::set_error(MYQL_ERR_UNSUPPORTED, "MLMC is not built yet");
}
