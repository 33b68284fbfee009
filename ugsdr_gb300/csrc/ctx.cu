// Context lifetime and the small C entry points around it.
#include "internal.hpp"

using namespace ugsdr_gpu;

extern "C" {

int ugsdr_ctx_create(int device, ugsdr_ctx** out) {
	if (!out)
		return UGSDR_E_INVALID;
	*out = nullptr;
	auto* ctx = new ugsdr_ctx();
	const int st = guarded(ctx, [&] {
		int count = 0;
		UG_CUDA(cudaGetDeviceCount(&count));
		require(device >= 0 && device < count, "no CUDA device " + std::to_string(device));
		ctx->device = device;
		UG_CUDA(cudaSetDevice(device));
		UG_CUDA(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
		ctx->stream = ctx->own_stream;
		UG_CUDA(cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device));
		int optin = 0;
		UG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
		ctx->smem_optin = static_cast<size_t>(optin);
		get_lut(ctx);
	});
	if (st != UGSDR_OK) {
		// keep the message reachable through a static buffer for the caller
		static thread_local std::string msg;
		msg = ctx->last_error;
		if (ctx->own_stream)
			cudaStreamDestroy(ctx->own_stream);
		delete ctx;
		return st;
	}
	*out = ctx;
	return UGSDR_OK;
}

int ugsdr_ctx_destroy(ugsdr_ctx* ctx) {
	if (!ctx)
		return UGSDR_E_INVALID;
	cudaSetDevice(ctx->device);
	cudaStreamSynchronize(ctx->stream);
	if (ctx->copy_stream) {
		cudaStreamSynchronize(ctx->copy_stream);
		cudaStreamDestroy(ctx->copy_stream);
	}
	for (int i = 0; i < 2; ++i) {
		if (ctx->slot_copied[i])
			cudaEventDestroy(ctx->slot_copied[i]);
		if (ctx->slot_used[i])
			cudaEventDestroy(ctx->slot_used[i]);
	}
	if (ctx->own_stream)
		cudaStreamDestroy(ctx->own_stream);
	delete ctx;
	return UGSDR_OK;
}

int ugsdr_ctx_set_stream(ugsdr_ctx* ctx, void* cuda_stream) {
	if (!ctx)
		return UGSDR_E_INVALID;
	std::lock_guard<std::mutex> lock(ctx->mutex);
	ctx->stream = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : ctx->own_stream;
	return UGSDR_OK;
}

int ugsdr_ctx_synchronize(ugsdr_ctx* ctx) {
	if (!ctx)
		return UGSDR_E_INVALID;
	return guarded(ctx, [&] { UG_CUDA(cudaStreamSynchronize(ctx->stream)); });
}

const char* ugsdr_last_error(const ugsdr_ctx* ctx) {
	if (!ctx)
		return "null context";
	return ctx->last_error.c_str();
}

int ugsdr_ctx_launch_count(const ugsdr_ctx* ctx, uint64_t* count) {
	if (!ctx || !count)
		return UGSDR_E_INVALID;
	*count = ctx->launches.load();
	return UGSDR_OK;
}
}

extern "C" {
int ugsdr_ctx_enable_timing(ugsdr_ctx* ctx, int on) {
	if (!ctx)
		return UGSDR_E_INVALID;
	std::lock_guard<std::mutex> lock(ctx->mutex);
	ctx->timing = on != 0;
	return UGSDR_OK;
}

int ugsdr_ctx_kernel_time(ugsdr_ctx* ctx, const char* kernel, uint64_t* launches, double* total_ms) {
	if (!ctx || !kernel || !launches || !total_ms)
		return UGSDR_E_INVALID;
	std::lock_guard<std::mutex> lock(ctx->mutex);
	return guarded(ctx, [&] {
		for (auto& t : ctx->timed) {
			UG_CUDA(cudaEventSynchronize(t.stop));
			float ms = 0.f;
			UG_CUDA(cudaEventElapsedTime(&ms, t.start, t.stop));
			auto& tot = ctx->kernel_totals[t.name];
			tot.first += 1;
			tot.second += ms;
			cudaEventDestroy(t.start);
			cudaEventDestroy(t.stop);
		}
		ctx->timed.clear();
		auto it = ctx->kernel_totals.find(kernel);
		*launches = it == ctx->kernel_totals.end() ? 0 : it->second.first;
		*total_ms = it == ctx->kernel_totals.end() ? 0.0 : it->second.second;
	});
}

int ugsdr_ctx_reset_timing(ugsdr_ctx* ctx) {
	if (!ctx)
		return UGSDR_E_INVALID;
	std::lock_guard<std::mutex> lock(ctx->mutex);
	return guarded(ctx, [&] {
		for (auto& t : ctx->timed) {
			cudaEventSynchronize(t.stop);
			cudaEventDestroy(t.start);
			cudaEventDestroy(t.stop);
		}
		ctx->timed.clear();
		ctx->kernel_totals.clear();
	});
}
}
