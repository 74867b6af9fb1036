/* IXAHWave.h (shim) -- see XA_ini.h.  TEST INFRASTRUCTURE ONLY. */
#pragma once
#include "XA_ini.h"
