// Launchers of the derived-field kernel (dg_output.cuh) for every precision and basis.
#include "dg_output.cuh"

namespace hermes {
bool derived_launcher(int precision, int nb, DerivedFn* out) {
    if (precision == 64 && nb == 4) *out = &derived_launch<double, 4, 2>;
    else if (precision == 64 && nb == 8) *out = &derived_launch<double, 8, 2>;
    else if (precision == 64 && nb == 10) *out = &derived_launch<double, 10, 3>;
    else if (precision == 32 && nb == 4) *out = &derived_launch<float, 4, 2>;
    else if (precision == 32 && nb == 8) *out = &derived_launch<float, 8, 2>;
    else if (precision == 32 && nb == 10) *out = &derived_launch<float, 10, 3>;
    else return false;
    return true;
}
}  // namespace hermes
