// Stage ids for the per-stage event timer (see prof.cu).
#pragma once
#include "common.cuh"

enum {
  AGB_ST_GAP = 0,      // host time between launches (descriptor copies, syncs)
  AGB_ST_SETUP = 1,
  AGB_ST_CONTRACT = 2,
  AGB_ST_GRAM = 3,
  AGB_ST_TRIDIAG = 4,
  AGB_ST_BISECT = 5,
  AGB_ST_INVIT = 6,
  AGB_ST_CLUSTER = 7,
  AGB_ST_BACKTRANS = 8,
  AGB_ST_POLISH = 9,
  AGB_ST_AV = 10,
  AGB_ST_RANK = 11,
  AGB_ST_SCATTER = 12,
  AGB_PROF_NSTAGES = 16
};

void prof_mark(int stage, cudaStream_t s);
