// Sky-loop kernel variants for 3 detectors (see skyloop_kernel.cuh).
#include "skyloop_kernel.cuh"

namespace pgw {

KernelFn pick_kernel_i3(int n_ifo, int lps, int minb, bool fast) {
  switch (n_ifo) {
    case 3: return pick_variant<3>(lps, minb, fast);
    default: return nullptr;
  }
}

}  // namespace pgw
