// Radix planning shared by the engine and the host-side FFT check.
#pragma once

#include <algorithm>
#include <functional>
#include <vector>

namespace ugsdr_gpu {
	// Radices the kernels dispatch on (butterfly_dispatch in fft_core.cuh).
	inline bool radix_supported(int r) {
		static const int list[] = {2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 16, 17, 19, 20, 23, 25, 27, 29, 31, 32};
		for (int x : list)
			if (x == r)
				return true;
		return false;
	}

	// Factor n into supported radices with the fewest passes, radices
	// non-increasing (one representative per multiset).  Empty on failure.
	inline bool plan_radices(int n, std::vector<int>& best) {
		std::vector<int> cur;
		best.clear();
		std::function<void(int)> dfs = [&](int rest) {
			if (!best.empty() && cur.size() >= best.size())
				return;
			if (rest == 1) {
				best = cur;
				return;
			}
			for (int r = 32; r >= 2; --r) {
				if (rest % r || !radix_supported(r))
					continue;
				if (!cur.empty() && r > cur.back())
					continue;
				cur.push_back(r);
				dfs(rest / r);
				cur.pop_back();
			}
		};
		dfs(n);
		// Odd radices first: the first Stockham pass stores with a stride of R
		// elements, which is conflict-free in shared memory only for odd R.
		std::stable_sort(best.begin(), best.end(), [](int a, int b) { return (a & 1) > (b & 1); });
		return !best.empty();
	}
}
