// Forwarding header of the oracle's TBB-API shim.
#pragma once
#include "tbb_shim_core.h"
