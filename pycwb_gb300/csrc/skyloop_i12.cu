// Sky-loop kernel variants for 1 and 2 detectors (see skyloop_kernel.cuh).
#include "skyloop_kernel.cuh"

namespace pgw {

KernelFn pick_kernel_i12(int n_ifo, int lps, int minb, bool fast) {
  switch (n_ifo) {
    case 1: return pick_variant<1>(lps, minb, fast);
    case 2: return pick_variant<2>(lps, minb, fast);
    default: return nullptr;
  }
}

}  // namespace pgw
