// Empty stand-in of <cusp/print.h> for the CPU build of the reference
// (test infrastructure only).
#pragma once
namespace cusp {
template <typename T>
void print(const T&) {}
}  // namespace cusp
