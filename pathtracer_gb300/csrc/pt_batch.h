// pt_batch.h -- batched rendering in one CUDA-graph launch and the launch
// autotuner (pt_batch.cpp).
#pragma once
#include "pt_host.h"

namespace pt {

// films: host films receiving each job's mean (may be null).  targets: when
// given, device films the samples are ADDED onto instead (no readback).
void render_batch(Context *c, const pt_job_desc *jobs, int n, float **films, pt_stats *stats,
                  float **targets = nullptr);
void autotune(Context *c, const pt_job_desc *jobs, int n, pt_tuning *out);

}  // namespace pt
