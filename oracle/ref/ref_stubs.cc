// Definitions the reference's bin_packer_2d.cc links against but that the
// pinning never reaches: only its DrawPackedRects (not called here) asks for
// random colours, and image_util.cc, which defines them, needs parts of Eigen
// the shim does not provide.  TEST INFRASTRUCTURE ONLY.
#include <cstdio>
#include <cstdlib>

#include "ugu/util/image_util.h"

namespace ugu {

std::vector<Eigen::Vector3f> GenRandomColors(int32_t, float, float, size_t) {
  std::fprintf(stderr, "ref_stubs: GenRandomColors is not part of the pinned code\n");
  std::abort();
}

}  // namespace ugu
