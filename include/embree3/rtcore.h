/* Drop-in include path: programs that include <embree3/rtcore.h> get the
   GB300 library's declarations. */
#pragma once
#include "../rtcore_gb300.h"
