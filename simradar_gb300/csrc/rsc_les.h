/*
 * rsc_les.h -- what the device side (rsc.cu) needs from an LES frame source
 * (rsc_les.cpp): a frame's raw planes in host memory, held while a copy out
 * of them is in flight.
 */
#ifndef SIMRADAR_GB300_RSC_LES_H
#define SIMRADAR_GB300_RSC_LES_H

#include <cuda_runtime.h>
#include <stddef.h>

#include "../../include/rsc.h"

namespace rscles {

/* A frame held by the caller: `planes` are the u, v, w, p, t planes as the
 * file stores them (nn floats each, unscaled), `nn` the cells per plane. */
struct Held {
    const float *planes = nullptr;
    size_t nn = 0;
    float time = 0.0f;
    int entry = -1;
};

/* Frame `frame` in one of the source's buffers (read now unless the thread
 * has it), held until release(); the frame after it is read ahead. */
int acquire(rsc_les_source *src, uint32_t frame, Held *out, const char **why);
/* Page-lock the held buffer for asynchronous copies (once per buffer). */
int pin(rsc_les_source *src, const Held &h, const char **why);
/* Give the buffer back.  With a copy stream, the buffer is not refilled
 * before the work queued on that stream so far (the copy out of it) is done. */
void release(rsc_les_source *src, const Held &h, cudaStream_t copy_stream);
const rsc_les_info &info(const rsc_les_source *src);

}  // namespace rscles

#endif
