// Stand-in for miniply.h: the reference includes it from plymesh.hpp; the
// triangle test built from shape.cpp reads no PLY file (test infrastructure).
#pragma once
