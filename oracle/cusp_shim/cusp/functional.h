// Empty stand-in of <cusp/functional.h> for the CPU build of the reference
// (test infrastructure only).
#pragma once
