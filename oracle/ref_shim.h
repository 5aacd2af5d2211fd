/* ref_shim.h -- force-included (g++ -include) when the reference kd-tree
 * builder is compiled from its own sources, where they lie, by
 * oracle/build_ref.sh.  TEST INFRASTRUCTURE ONLY: nothing in the product
 * links the binary this produces.
 *
 * The reference is an MSVC project.  Three things keep its builder
 * translation units (Kd-treeConstructor.cpp, Kd-treeConverter.cpp,
 * MyMathUtility.cpp) from compiling with g++ on Linux; each is handled here
 * without editing a reference file:
 *   1. __declspec(align(16)) on TriAccel (Kd-treeConverter.h:205) and
 *      _aligned_malloc: mapped to GCC equivalents.
 *   2. The MSVC-only constructor spelling `struct _SplitCost(void):`
 *      (Kd-treeConstructor.h:46).  A function-like macro named _SplitCost only
 *      expands where the tag is followed by '(' (that one line), turning it
 *      into `struct _SplitCostFwd; _SplitCost(void):` -- a nested forward
 *      declaration followed by an ordinary constructor.  The macro does not
 *      re-expand inside its own replacement.
 *   3. The committed configuration is PRIMITIVE_TYPE 0 (triangles,
 *      Kd-treeConverter.h:22).  The hybrid Gaussian kd-tree is
 *      PRIMITIVE_TYPE 2 (ELLIPSOID_BY_TRI).  The header is included here
 *      first (it is #pragma once), then the mode macros it derived from the
 *      committed value are re-set to what PRIMITIVE_TYPE 2 derives:
 *      COUNT_BY_GID 1 (Kd-treeConverter.h:39,66-69) and SECONDARY_RAY 1
 *      (:26,33-36).  Every later `#if PRIMITIVE_TYPE == ...` in the builder
 *      sources then sees 2.  KdTree keeps the TRI-only tri_accel_list
 *      member (:291-293); all translation units see the same layout and the
 *      builder never touches it in mode 2.
 *   4. uint32_t is used without <cstdint> (Gaussian.h:6).
 */
#pragma once
#include <stdlib.h>
#include <stdint.h>
#include <float.h>

#define __declspec(x)
#define _aligned_malloc(sz, al) aligned_alloc((al), (sz))
#define _aligned_free free
#define _SplitCost(v) _SplitCostFwd; _SplitCost(v)

#include "Kd-treeConverter.h"

#undef PRIMITIVE_TYPE
#define PRIMITIVE_TYPE 2
#undef COUNT_BY_GID
#define COUNT_BY_GID 1
#undef SECONDARY_RAY
#define SECONDARY_RAY 1
