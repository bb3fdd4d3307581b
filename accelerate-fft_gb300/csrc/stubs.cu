// Entry points of subsystems that are not built yet report
// GBFFT_ERR_UNSUPPORTED so the C ABI stays complete.
#include "gbfft.h"
#include "plan_internal.h"

namespace gbfft {
int build_split_plan(gbfft_plan*) { return GBFFT_ERR_UNSUPPORTED; }
}  // namespace gbfft

extern "C" {
int gbfft_specconv_plan_create(gbfft_specconv_plan** out, int64_t, int64_t, int64_t, int64_t, int) {
  if (out) *out = nullptr;
  return GBFFT_ERR_UNSUPPORTED;
}
int gbfft_specconv_fwd(const gbfft_specconv_plan*, const void*, const void*, void*, void*) {
  return GBFFT_ERR_UNSUPPORTED;
}
int gbfft_specconv_bwd(const gbfft_specconv_plan*, const void*, const void*, const void*, void*, void*,
                       void*) {
  return GBFFT_ERR_UNSUPPORTED;
}
int gbfft_specconv_plan_destroy(gbfft_specconv_plan*) { return GBFFT_OK; }
}
