// FP64 instantiation of the stage kernels. Built with --fmad=false so that every
// operation rounds exactly like the reference's scalar FP64 code (bit-exact parity).
#define ATHG_LAUNCH_IMPL
#include "athg_launch.cuh"
namespace athg {
template struct Launcher<double>;
}
