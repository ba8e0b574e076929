// Stepper instantiations for 1D (p = 1..4).
#include "spd_stepper.cuh"

namespace spd_host {
StepperBase* make_stepper_d1(int P) { return make_stepper_for<1>(P); }
}  // namespace spd_host
