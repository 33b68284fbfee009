// Project-written stand-in for boost::iostreams::mapped_file_source, enough
// for the reference's src/signal_parameters.hpp:44-84 to compile (Boost is
// not installed here).  TEST / INTEGRATION-CHECK INFRASTRUCTURE ONLY: reads
// the whole file into memory instead of mapping it.
#pragma once

#include <cstddef>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>

namespace boost {
	namespace iostreams {
		class mapped_file_source {
			std::vector<char> bytes_;
			bool open_ = false;

		public:
			void open(const std::string& path) {
				std::ifstream f(path, std::ios::binary);
				open_ = static_cast<bool>(f);
				if (open_)
					bytes_.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
			}
			bool is_open() const { return open_; }
			const char* data() const { return bytes_.data(); }
			std::size_t size() const { return bytes_.size(); }
		};
	}
}
