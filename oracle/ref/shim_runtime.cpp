/* Definitions behind the host-only CUDA stand-in and the reference's profiler hooks
 * (profiler.h declares them; the profiler itself is not part of the host-only compile). */
#include <cuda_runtime.h>
#include <profiler.h>

thread_local dim3 threadIdx, blockIdx, blockDim, gridDim;

void ProfilerInitKernel(int) {}
void ProfilerPrepare(const char *) {}
void ProfilerBeginStep() {}
void ProfilerIncreaseStepIteration() {}
int ProfilerGetIterationsPassed() { return 0; }
double ProfilerGetStepInterval() { return 0; }
double ProfilerGetEvaluation(const char *) { return 0; }
void ProfilerEndStep() {}
void ProfilerFinish() {}
void ProfilerReport(int) {}
void ProfilerManualStart(const char *) {}
void ProfilerManualFinish() {}
void _ProfilerSetParticle(int, int) {}
