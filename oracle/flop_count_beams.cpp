// ORACLE — test infrastructure only.  eb_oracle_beams.cpp compiled over flop::Real for
// flop_count.cpp (the operation count of the restatement, not a second oracle).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "flop_real.hpp"
#define double flop::Real
#include "eb_oracle_beams.cpp"
#undef double
