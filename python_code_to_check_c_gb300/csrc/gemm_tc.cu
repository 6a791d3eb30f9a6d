// Tensor-core (tcgen05) backend for the large contractions of the mixed
// precision mode.
#include "engine.h"

namespace tdcc {

bool tc_available() { return false; }

}  // namespace tdcc
