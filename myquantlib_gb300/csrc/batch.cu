// batch.cu -- many pricing requests in one launch sequence (placeholder until
// the persistent work-queue kernel lands).
#include "engine.h"

extern "C" myql_status myql_mc_price_batch(myql_ctx *, const myql_mc_job *, size_t,
                                           double *const *, myql_mc_stats *) {
  return myql::set_error(MYQL_ERR_UNSUPPORTED, "batched pricing is not built yet");
}
