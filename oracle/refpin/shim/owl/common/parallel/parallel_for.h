// parallel_for.h -- TEST INFRASTRUCTURE ONLY: placeholder for owl's
// parallel-for header, which the reference includes but does not use on
// the code compiled into the pin harness.
#pragma once
#include "../owl-common.h"
