// Tracking correlator bank (placeholder until the bank kernel lands).
#include "internal.hpp"

using namespace ugsdr_gpu;

struct ugsdr_track_bank {
	ugsdr_ctx* ctx = nullptr;
};

extern "C" {
int ugsdr_track_create(ugsdr_ctx* ctx, const ugsdr_track_config*, const ugsdr_track_channel*, int, const float*, const int*, int,
	int, ugsdr_track_bank** bank) {
	if (bank)
		*bank = nullptr;
	if (ctx)
		ctx->last_error = "tracking bank not built";
	return UGSDR_E_UNSUPPORTED;
}
int ugsdr_track_run(ugsdr_track_bank*, const void*, int, int, size_t, int, ugsdr_track_output*) { return UGSDR_E_UNSUPPORTED; }
int ugsdr_track_destroy(ugsdr_track_bank* bank) {
	delete bank;
	return UGSDR_OK;
}
}
