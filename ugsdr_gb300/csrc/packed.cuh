// Decoders of the packed front-end capture formats (BBP DDC, NT1065 grabber)
// and a loader over every sample type for the kernels that take raw captures.
#pragma once

#include "acq_kernels.cuh"

namespace ugsdr_gpu {

	// Framing of a packed capture: samples per 1 ms epoch and, for BBP DDC,
	// bytes per epoch (8-byte header + samples + padding).
	struct PackedLayout {
		uint32_t spm = 0;
		uint32_t epoch_bytes = 0;
	};

	// BBP DDC sample i (helpers/BbpPackedSpan.hpp): byte (i mod spm) / 2 after
	// the epoch's 8-byte header; the even sample holds imag in bits 0-1 and
	// real in bits 2-3, the odd one bits 4-5 and 6-7; each signed 2-bit field
	// f is read as (f | 1), i.e. -1 when its top bit is set and +1 otherwise.
	__device__ __forceinline__ float2 decode_bbp(const unsigned char* base, uint64_t i, const PackedLayout& l) {
		const uint64_t e = i / l.spm;
		const uint32_t s = static_cast<uint32_t>(i - e * l.spm);
		const unsigned b = base[e * l.epoch_bytes + 8 + (s >> 1)];
		const unsigned sh = (s & 1u) << 2;
		return c2(((b >> (sh + 3)) & 1u) ? -1.f : 1.f, ((b >> (sh + 1)) & 1u) ? -1.f : 1.f);
	}

	// NT1065 sample i (helpers/NtlabPackedSpan.hpp): byte i, sign at bit
	// `offset`, magnitude above it: (2 sign - 1)(1 + 2 magnitude), real.
	__device__ __forceinline__ float2 decode_nt1065(const unsigned char* base, uint64_t i, int offset) {
		const unsigned b = base[i] >> offset;
		const int sign = static_cast<int>(b & 1u), mag = static_cast<int>((b >> 1) & 1u);
		return c2(static_cast<float>((2 * sign - 1) * (1 + 2 * mag)), 0.f);
	}

	template <int ST>
	__device__ __forceinline__ float2 load_any(const void* base, uint64_t i, const PackedLayout& l) {
		if constexpr (ST <= UGSDR_SAMPLES_RI8)
			return load_sample<ST>(base, i);
		else if constexpr (ST == UGSDR_SAMPLES_BBP_DDC)
			return decode_bbp(static_cast<const unsigned char*>(base), i, l);
		else
			return decode_nt1065(static_cast<const unsigned char*>(base), i, 6 - 2 * (ST - UGSDR_SAMPLES_NT1065_1));
	}

	// Any sample type -> complex float (runtime type; one pass, memory bound).
	static __global__ void __launch_bounds__(256) unpack_kernel(const void* in, int type, PackedLayout l, uint64_t n, float2* out) {
		const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
		for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n; i += stride) {
			float2 v;
			switch (type) {
			case UGSDR_SAMPLES_CF32: v = load_sample<UGSDR_SAMPLES_CF32>(in, i); break;
			case UGSDR_SAMPLES_CI8: v = load_sample<UGSDR_SAMPLES_CI8>(in, i); break;
			case UGSDR_SAMPLES_CI16: v = load_sample<UGSDR_SAMPLES_CI16>(in, i); break;
			case UGSDR_SAMPLES_RI8: v = load_sample<UGSDR_SAMPLES_RI8>(in, i); break;
			case UGSDR_SAMPLES_BBP_DDC: v = decode_bbp(static_cast<const unsigned char*>(in), i, l); break;
			default: v = decode_nt1065(static_cast<const unsigned char*>(in), i, 6 - 2 * (type - UGSDR_SAMPLES_NT1065_1)); break;
			}
			out[i] = v;
		}
	}
}
