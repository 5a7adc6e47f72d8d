// Stand-in for splash/utils/math_utils.hpp: included, not used, by the
// Stouffer kernel header.  Test infrastructure only.
#pragma once
#include <cmath>
