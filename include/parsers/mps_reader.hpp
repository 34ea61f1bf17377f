// Free-format MPS reader (NAME / ROWS / COLUMNS / RHS / BOUNDS, integer markers).
// Same entry point and row conversion as the reference's
// src/parsers/mps_reader.hpp:20 / mps_reader.cpp:65-355: each L row gets a +1
// slack column, each G row a -1 surplus column, slacks appended after the
// structural columns in row order; RANGES / SOS and unknown sections throw.
#pragma once

#include <string>

#include "core/problem.hpp"

namespace sankhya {
namespace parsers {

core::Model read_mps(const std::string& filename);

}  // namespace parsers
}  // namespace sankhya
