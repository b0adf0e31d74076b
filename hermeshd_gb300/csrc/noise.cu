// Launchers of the staged stochastic-stress kernels (dg_noise.cuh) for every precision and basis.
#include "dg_noise.cuh"

namespace hermes {
bool noise_launcher(int precision, int nb, NoiseFn* out) {
    if (precision == 64 && nb == 4) *out = &noise_launch<double, 4, 2>;
    else if (precision == 64 && nb == 8) *out = &noise_launch<double, 8, 2>;
    else if (precision == 64 && nb == 10) *out = &noise_launch<double, 10, 3>;
    else if (precision == 32 && nb == 4) *out = &noise_launch<float, 4, 2>;
    else if (precision == 32 && nb == 8) *out = &noise_launch<float, 8, 2>;
    else if (precision == 32 && nb == 10) *out = &noise_launch<float, 10, 3>;
    else return false;
    return true;
}
}  // namespace hermes
