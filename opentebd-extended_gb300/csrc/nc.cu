// nc.cu -- number-conserving (U(1) block-sparse) two-site update.
#include "tebd_internal.cuh"

namespace tebd {

int nc_alloc(tebd_handle *h) {
  h->nc_ws = nullptr;
  h->nc_ws_bytes = 0;
  return TEBD_OK;
}

void nc_free(tebd_handle *h) {
  if (h->nc_ws) cudaFree(h->nc_ws);
  h->nc_ws = nullptr;
}

int run_nc_batch(tebd_handle *h, int, const int *, double *) {
  return set_error(h, TEBD_ERR_STATE, "number-conserving update not built yet");
}

}  // namespace tebd
