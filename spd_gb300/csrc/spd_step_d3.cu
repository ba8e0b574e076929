// Stepper instantiations for 3D (p = 1..4).
#include "spd_stepper.cuh"

namespace spd_host {
StepperBase* make_stepper_d3(int P) { return make_stepper_for<3>(P); }
}  // namespace spd_host
