// Shared definitions of the fem2d_gb300 host library.
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>

#include "../../include/fem2d_gb300.h"

namespace fem2d {

// An error that carries one of the FEM2D_E_* status codes across the C ABI.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] inline void fail(int code, const std::string& msg) { throw Error(code, msg); }

void set_last_error(const std::string& msg);

}  // namespace fem2d
