// Empty stand-in of <cusp/transpose.h> for the CPU build of the reference
// (test infrastructure only).
#pragma once
