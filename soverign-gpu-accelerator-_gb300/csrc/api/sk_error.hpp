// Error plumbing of the C ABI: internal code throws sk_exception (or standard
// exceptions); every extern "C" entry converts them into SK_* codes and keeps the
// message for sk_last_error().
#pragma once

#include <stdexcept>
#include <string>

#include "core/sparse_matrix.hpp"

namespace sankhya {
namespace api {

struct sk_exception : std::runtime_error {
    int code;
    sk_exception(int c, const std::string& msg) : std::runtime_error(msg), code(c) {}
};

void set_error(const std::string& msg);
void clear_error();
int status_of_current_exception();
core::CSRMatrix pattern_csr(int m, int n, const int* row_ptrs, const int* col_idx);

}  // namespace api
}  // namespace sankhya
