/* Stand-in for the CUDA runtime header when the reference sources are compiled as host C++.
 * Test infrastructure only: everything the reference needs comes from gdref_prelude.h. */
#pragma once
#include "gdref_prelude.h"
