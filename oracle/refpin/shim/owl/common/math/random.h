// random.h -- TEST INFRASTRUCTURE ONLY: placeholder for owl's random-number
// header, which the reference includes but does not use on this path.
#pragma once
#include "vec.h"
