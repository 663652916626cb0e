// gbo_merge.h : the hit merge (gbo_merge.cu) for the engine, with work buffers kept between events.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gbopticks.h"

namespace gbo {

struct MergeScratch;
MergeScratch* merge_scratch_new();
void merge_scratch_free(MergeScratch* m);
int merge_hits(const gbo_sphoton* d_in, int64_t n, float time_window, gbo_sphoton* d_out, int64_t* num_out,
               cudaStream_t s, MergeScratch* scratch);

}  // namespace gbo
