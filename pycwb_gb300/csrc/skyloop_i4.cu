// Sky-loop kernel variants for 4 detectors (see skyloop_kernel.cuh).
#include "skyloop_kernel.cuh"

namespace pgw {

KernelFn pick_kernel_i4(int n_ifo, int lps, int minb, bool fast) {
  switch (n_ifo) {
    case 4: return pick_variant<4>(lps, minb, fast);
    default: return nullptr;
  }
}

}  // namespace pgw
