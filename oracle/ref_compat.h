/* Forced include for compiling the reference's CPU sources with g++ 13:
 * GPBlocks.cpp:251 calls an unqualified max() without including <algorithm>. */
#include <algorithm>
#include <cstdint>
using std::max;
