/*
 * ORACLE -- test infrastructure, not part of the product.
 *
 * A plain-C restatement of the reference (thomgrand/torch_kdtree) CPU path:
 *   - orc_build_*  : createKDTree / createPartitionRecursive / compMedian
 *                    (src/kdtree.hpp:392-534)
 *   - orc_query_*  : KDTreeKNNSearch + searchKDTreeIteratively + the
 *                    TreeTraversal tag walk (src/kdtree.cpp:16-110,164-194;
 *                    src/kdtree.hpp:225-379, 546-692; src/nndistance.hpp)
 *   - orc_brute_*  : exhaustive k smallest (distance, original index) pairs
 *                    with the same distance arithmetic (the canonical answer
 *                    of the GPU kernels).
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this library, and only as a checker or a timed CPU baseline.
 *
 * Parity of this restatement is pinned against the reference itself:
 * tests/golden/make_golden.py runs the reference's own sources (compiled by
 * oracle/Makefile into oracle/_ref/) and the fixtures it writes are checked
 * against this file by tests/test_oracle.py.
 *
 * Must be compiled with -ffp-contract=off: the reference's distance is
 * ((0 + d0*d0) + d1*d1) + d2*d2 with every operation rounded separately.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_TREE_MAX_D 8
#define ORC_MAX_D 128

enum { TAG_NONE = 0, TAG_LEFT = 1, TAG_RIGHT = 2, TAG_BOTH = 3 };
enum { DIR_UP = 0, DIR_LEFT = 1, DIR_RIGHT = 2, DIR_DONE = 3 };

#define OT float
#define OSFX f32
#include "kdtree_oracle.inc"
#undef OT
#undef OSFX

#define OT double
#define OSFX f64
#include "kdtree_oracle.inc"
#undef OT
#undef OSFX

int orc_version(void) { return 1; }
