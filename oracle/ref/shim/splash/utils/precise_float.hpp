// Stand-in for splash/utils/precise_float.hpp: included, not used, by the
// Stouffer and CLR kernel headers.  Test infrastructure only.
#pragma once
