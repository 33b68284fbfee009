// Digital front end on the device: Mixer::Translate at the input rate followed
// by SequentialResampler, with the reference's float rounding.
#pragma once

#include "packed.cuh"

namespace ugsdr_gpu {

	// SequentialResampler::Process (resample/resampler.hpp:39-46) for integer
	// rates: SequentialUpsampler to lcm(new, old) samples (upsampler.hpp:30-37,
	// upsampled i reads input floor(i / L), L = lcm / old), then Accumulator
	// (decimator.hpp:53-69): output k is the float sum, in index order, of
	// upsampled [k M, (k+1) M), M = lcm / new, zero-padded past `up`, divided
	// by M.  The std::div names are swapped there ([rem, quot]), so a length
	// that M does not divide is padded to the next multiple instead of cut.
	struct ResamplePlan {
		uint64_t l;   // upsampling factor lcm / old
		uint64_t m;   // boxcar length lcm / new
		uint64_t up;  // upsampled length l * n_in
		uint64_t n_out;
	};

	// One output sample.  `load(j)` returns input j.  Each input is added as
	// many times as the boxcar covers its ZOH run, one float add at a time:
	// that repeats the reference's sequential sum bit for bit (padding zeros
	// change nothing: the sum starts at +0 and x + 0 == x).
	template <typename Load>
	__device__ __forceinline__ float2 resample_point(uint64_t k, const ResamplePlan& r, Load load) {
		if (r.m == 1)
			return load(k / r.l);  // Accumulator returns early for ratio 1
		const uint64_t i0 = k * r.m;
		const uint64_t i1 = min(i0 + r.m, r.up);
		float ax = 0.f, ay = 0.f;
		uint64_t i = i0;
		uint64_t j = i0 / r.l;
		while (i < i1) {
			const uint64_t stop = min((j + 1) * r.l, i1);
			const float2 v = load(j);
			for (uint64_t t = i; t < stop; ++t) {
				ax = __fadd_rn(ax, v.x);
				ay = __fadd_rn(ay, v.y);
			}
			i = stop;
			++j;
		}
		const float mf = static_cast<float>(r.m);
		return c2(__fdiv_rn(ax, mf), __fdiv_rn(ay, mf));
	}

	struct FrontEndParams {
		const void* samples;   // n_in input samples of the job's sample type
		PackedLayout layout;   // packed types: framing
		uint64_t n_in;
		ResamplePlan rs;
		uint32_t fe_adder;     // Translate(signal, fs_in, f) adder
		int fe_on;
		const float* lut;
		float2* out;           // n outputs
		uint64_t n;
	};

	// Decode (packed formats), Translate at the input rate (fse.hpp:289, 312:
	// phase 0 at input sample 0), then resample (fse.hpp:290-291, 313-314),
	// for the first p.n outputs.
	template <int ST>
	__global__ void __launch_bounds__(256) front_end_kernel(FrontEndParams p) {
		const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
		for (uint64_t k = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; k < p.n; k += stride) {
			p.out[k] = resample_point(k, p.rs, [&](uint64_t j) {
				float2 v = load_any<ST>(p.samples, j, p.layout);
				if (p.fe_on)
					v = table_mix(v, j, p.fe_adder, 0u, p.lut);
				return v;
			});
		}
	}
}
