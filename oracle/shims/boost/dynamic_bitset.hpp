// Project-written stand-in for boost::dynamic_bitset, enough for the
// reference's src/ephemeris/Ephemeris.hpp:13-21 (bin2dec: construct with a
// size, assign bits through operator[], read back with to_ulong) to compile
// (Boost is not installed here).  ORACLE / TEST INFRASTRUCTURE ONLY.
#pragma once

#include <cstddef>
#include <stdexcept>
#include <vector>

namespace boost {
	class dynamic_bitset {
	public:
		class reference {
		public:
			reference(std::vector<bool>& bits, std::size_t pos) : bits_(bits), pos_(pos) {}
			template <typename T>
			reference& operator=(const T& value) {
				bits_[pos_] = static_cast<bool>(value);
				return *this;
			}
			operator bool() const { return bits_[pos_]; }

		private:
			std::vector<bool>& bits_;
			std::size_t pos_;
		};

		dynamic_bitset(std::size_t n, unsigned long value) : bits_(n) {
			for (std::size_t i = 0; i < n && i < 8 * sizeof(value); ++i)
				bits_[i] = (value >> i) & 1ul;
		}

		reference operator[](std::size_t pos) { return reference(bits_, pos); }
		bool operator[](std::size_t pos) const { return bits_[pos]; }
		std::size_t size() const { return bits_.size(); }

		// bit i is worth 2^i; like Boost, throws when a set bit does not fit
		unsigned long to_ulong() const {
			unsigned long out = 0;
			for (std::size_t i = 0; i < bits_.size(); ++i) {
				if (!bits_[i])
					continue;
				if (i >= 8 * sizeof(out))
					throw std::overflow_error("dynamic_bitset::to_ulong overflow");
				out |= 1ul << i;
			}
			return out;
		}

	private:
		std::vector<bool> bits_;
	};
}
