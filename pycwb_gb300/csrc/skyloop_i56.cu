// Sky-loop kernel variants for 5 and 6 detectors (see skyloop_kernel.cuh).
#include "skyloop_kernel.cuh"

namespace pgw {

KernelFn pick_kernel_i56(int n_ifo, int lps, int minb, bool fast) {
  switch (n_ifo) {
    case 5: return pick_variant<5>(lps, minb, fast);
    case 6: return pick_variant<6>(lps, minb, fast);
    default: return nullptr;
  }
}

}  // namespace pgw
