// ssfft_large.cu -- multi-pass (four-step) transforms for sizes beyond one CTA.
#include "ssfft_host.h"

namespace ssfft {

struct LargePlan {
	int unused = 0;
};

ssfft_status plan_build_large(Plan *) { return SSFFT_ERR_UNSUPPORTED; }

ssfft_status launch_large(Plan *, int, const void *, void *, size_t, cudaStream_t) { return SSFFT_ERR_UNSUPPORTED; }

void large_release(LargePlan *lp) { delete lp; }

}  // namespace ssfft
