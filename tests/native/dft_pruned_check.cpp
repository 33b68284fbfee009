// CPU check of the pruned register DFTs (fft_core.cuh DftPruned): for every
// radix of the acquisition plans and every count NZ of live leading inputs,
// DftPruned<R, INV, NZ> on v[0..NZ) equals Dft<R, INV> on the zero-filled
// input, value for value (an exact zero may differ in sign only, which ==
// ignores).  Built with g++ (the DFT bodies are __host__ __device__) and
// -ffp-contract=off so both sides round the same way.  Prints "ok" and
// exits 0, or names the first mismatch and exits 1.
#include <cstdio>
#include <cstdlib>
#include <random>

#include "fft_core.cuh"

using namespace ugsdr_gpu;

static int failures = 0;

template <int R, bool INV, int NZ>
void check_one(std::mt19937& rng) {
	std::uniform_real_distribution<float> u(-1.f, 1.f);
	for (int trial = 0; trial < 20; ++trial) {
		float2 full[R], pruned[R];
		for (int i = 0; i < R; ++i) {
			full[i] = i < NZ ? c2(u(rng), u(rng)) : c2(0.f, 0.f);
			pruned[i] = i < NZ ? full[i] : c2(1e30f, -1e30f);  // never read
		}
		Dft<R, INV>::run(full);
		DftPruned<R, INV, NZ>::run(pruned);
		for (int i = 0; i < R; ++i) {
			if (!(full[i].x == pruned[i].x && full[i].y == pruned[i].y)) {
				if (failures++ < 10)
					std::printf("R=%d INV=%d NZ=%d out %d: %.9g%+.9gi vs %.9g%+.9gi\n", R, int(INV), NZ, i, full[i].x, full[i].y,
						pruned[i].x, pruned[i].y);
				return;
			}
		}
	}
}

template <int R, bool INV>
void check_radix(std::mt19937& rng) {
	static_for<1, R + 1>([&](auto nz) { check_one<R, INV, decltype(nz)::value>(rng); });
}

template <int R>
void check_both(std::mt19937& rng) {
	check_radix<R, false>(rng);
	check_radix<R, true>(rng);
}

int main() {
	std::mt19937 rng(7);
	check_both<2>(rng);
	check_both<3>(rng);
	check_both<4>(rng);
	check_both<5>(rng);
	check_both<8>(rng);
	check_both<10>(rng);
	check_both<16>(rng);
	check_both<20>(rng);
	check_both<25>(rng);
	if (failures) {
		std::printf("%d mismatches\n", failures);
		return 1;
	}
	std::printf("ok\n");
	return 0;
}
