// ppl.h -- empty stand-in for MSVC's Parallel Patterns Library header,
// which the reference's BVH includes but only uses in commented-out code.
#pragma once
