// Reference build shim (test infrastructure): see shim_splines.h.
#pragma once
#include "shim_splines.h"
