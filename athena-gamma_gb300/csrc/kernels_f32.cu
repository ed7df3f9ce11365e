// FP32 instantiation of the stage kernels (mixed path: FP32 reconstruction and
// Riemann fluxes, FP64 conserved state, face field and CT update).
#define ATHG_LAUNCH_IMPL
#define ATHG_MARCH_MIN_BLOCKS 5
#include "athg_launch.cuh"
namespace athg {
template struct Launcher<float>;
}
