/* Force-included into OpenVort's octree.c when the reference library is
 * built for parity checks: octree_init leaves `children[8]` uninitialised
 * (octree.c:26-34) and the recursion reads them, so every allocation in that
 * file is zero-filled.  The reference sources are not edited. */
#include <stdlib.h>
#define malloc(n) calloc(1, (n))
