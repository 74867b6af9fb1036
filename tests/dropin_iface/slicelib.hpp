// slicelib.hpp -- stand-in for the two pieces of the reference's slicelib.hpp
// that the autoslic drop-in uses: the param[] offsets of the grid size
// (TemsimLibrary/slicelib.hpp:210-211) and ToInt (slicelib.hpp:260).
// TEST ONLY.
#ifndef MSK_TEST_SLICELIB_HPP
#define MSK_TEST_SLICELIB_HPP

enum { pNX = 104, pNY = 105 };

inline int ToInt(const float x) { return int(x + 0.1F); }

#endif
