// Library-internal access to a handle's step machinery, for the serving
// engine (server.cu).  Not part of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include "actflow.h"

namespace af {

// Energy-ring capacity of a handle: the largest chunk handle_enqueue_chunk takes.
int handle_ring_capacity();

// Enqueue k steps on the handle's stream without waiting: reset the ring
// index, replay the step graph k times, copy the k energies to energy_host
// (nullptr: not copied) and the handle's scalars (64 bytes: mean flow, step
// counter, NaN step) to scalars_host, then record `done`.  The host buffers
// should be pinned for the copies to run asynchronously; they are written when
// `done` has completed.
am_status handle_enqueue_chunk(am_handle *h, int k, double *energy_host, void *scalars_host, cudaEvent_t done);

// The stream the handle's work runs on.
cudaStream_t handle_stream(const am_handle *h);

}  // namespace af
