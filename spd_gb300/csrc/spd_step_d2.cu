// Stepper instantiations for 2D (p = 1..4).
#include "spd_stepper.cuh"

namespace spd_host {
StepperBase* make_stepper_d2(int P) { return make_stepper_for<2>(P); }
}  // namespace spd_host
