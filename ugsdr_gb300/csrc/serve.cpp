// Serving loop (placeholder until the server lands).
#include "internal.hpp"

struct ugsdr_server {
	ugsdr_ctx* ctx = nullptr;
};

extern "C" {
int ugsdr_server_create(ugsdr_ctx* ctx, const ugsdr_server_config*, ugsdr_server** server) {
	if (server)
		*server = nullptr;
	if (ctx)
		ctx->last_error = "server not built";
	return UGSDR_E_UNSUPPORTED;
}
int ugsdr_server_submit(ugsdr_server*, const ugsdr_acq_job*, uint64_t*) { return UGSDR_E_UNSUPPORTED; }
int ugsdr_server_poll(ugsdr_server*, uint64_t, ugsdr_acq_result*, int*) { return UGSDR_E_UNSUPPORTED; }
int ugsdr_server_drain(ugsdr_server*) { return UGSDR_E_UNSUPPORTED; }
int ugsdr_server_destroy(ugsdr_server* server) {
	delete server;
	return UGSDR_OK;
}
}
