// Empty stand-in of <cusp/multiply.h> for the CPU build of the reference
// (test infrastructure only).
#pragma once
