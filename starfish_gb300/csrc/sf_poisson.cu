// sf_poisson.cu -- placeholder until the Poisson solver lands.
#include "sf_internal.h"

void sf_poisson_destroy_internal(sf_ctx*) {}
int sf_poisson_get_field_internal(sf_ctx* ctx, int, double*) {
  ctx->err = "field solver not initialised";
  return SF_ERR_STATE;
}
