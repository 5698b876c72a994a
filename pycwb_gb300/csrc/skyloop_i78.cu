// Sky-loop kernel variants for 7 and 8 detectors (see skyloop_kernel.cuh).
#include "skyloop_kernel.cuh"

namespace pgw {

KernelFn pick_kernel_i78(int n_ifo, int lps, int minb, bool fast) {
  switch (n_ifo) {
    case 7: return pick_variant<7>(lps, minb, fast);
    case 8: return pick_variant<8>(lps, minb, fast);
    default: return nullptr;
  }
}

}  // namespace pgw
