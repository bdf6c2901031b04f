#include <stdio.h>
// Per-stage CUDA-event timing of the two-site pipeline.  When enabled, each
// stage boundary records an event on the launching stream; agb_prof_end sums
// the elapsed time between consecutive marks per stage.  Events are created
// once (no device memory is allocated).
#include <vector>

#include "prof.cuh"

namespace {
struct ProfState {
  bool on = false;
  int n = 0;
  std::vector<cudaEvent_t> ev;
  std::vector<int> stage;
};
ProfState g_prof;
long long g_launches = 0;
}  // namespace

void agb_note_launch() { ++g_launches; }

extern "C" long long agb_launch_count(void) { return g_launches; }

// The most recent failed launch check: "file:line: cudaErrorName (description)".
static char g_last_error[256] = "";

void agb_note_error(const char* file, int line, cudaError_t e) {
  const char* base = file;
  for (const char* p = file; *p; ++p)
    if (*p == '/') base = p + 1;
  snprintf(g_last_error, sizeof(g_last_error), "%s:%d: %s (%s)", base, line, cudaGetErrorName(e),
           cudaGetErrorString(e));
}

extern "C" const char* agb_last_error(void) { return g_last_error; }

void prof_mark(int stage, cudaStream_t s) {
  if (!g_prof.on) return;
  if (g_prof.n >= (int)g_prof.ev.size()) return;
  cudaEventRecord(g_prof.ev[g_prof.n], s);
  g_prof.stage[g_prof.n] = stage;
  ++g_prof.n;
}

extern "C" int agb_prof_begin(int capacity) {
  if (capacity <= 0) return AGB_ERR_ARG;
  while ((int)g_prof.ev.size() < capacity) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return AGB_ERR_CUDA;
    g_prof.ev.push_back(e);
  }
  g_prof.stage.resize(g_prof.ev.size());
  g_prof.n = 0;
  g_prof.on = true;
  return AGB_OK;
}

extern "C" int agb_prof_end(double* ms_per_stage, int* marks_per_stage, int nstages) {
  g_prof.on = false;
  if (!ms_per_stage || !marks_per_stage || nstages < AGB_PROF_NSTAGES) return AGB_ERR_ARG;
  for (int i = 0; i < nstages; ++i) {
    ms_per_stage[i] = 0;
    marks_per_stage[i] = 0;
  }
  if (g_prof.n == 0) return AGB_OK;
  if (cudaEventSynchronize(g_prof.ev[g_prof.n - 1]) != cudaSuccess) return AGB_ERR_CUDA;
  for (int i = 0; i + 1 < g_prof.n; ++i) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, g_prof.ev[i], g_prof.ev[i + 1]) != cudaSuccess) return AGB_ERR_CUDA;
    const int st = g_prof.stage[i];
    ms_per_stage[st] += ms;
    marks_per_stage[st] += 1;
  }
  g_prof.n = 0;
  return AGB_OK;
}
