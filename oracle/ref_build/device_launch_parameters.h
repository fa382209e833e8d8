/* Stand-in for the CUDA launch-parameter header (blockIdx & co. live in gdref_prelude.h).
 * Test infrastructure only. */
#pragma once
#include "gdref_prelude.h"
