// Stand-in header for the reference's LBVH sources (test infrastructure).
#pragma once
#include "rtcore.h"
