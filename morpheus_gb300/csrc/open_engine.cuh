// Continuous batching of Basefold openings (lockstep.cu).
//
// An open engine is one host thread with one stream that keeps a set of openings in flight.
// Openings join the set whenever they are submitted (at the next step boundary) and leave it
// when their queries are gathered; each step advances every opening in the set by one round
// of open_ext2 (goldilocks-cuda-rs/src/basefold.rs:578-870), whatever round each is in, with one
// launch per kernel kind for all of them (ragged segment tables) and one host round trip.
// Each opening's transcript is its own, so its proof does not depend on the others in the set.
#pragma once
#include <functional>
#include <string>
#include <vector>

#include "../../include/goldilocks_cuda_wrapper.h"
#include "basefold.cuh"

namespace gb {

struct OpenTask {
    BfCommitment* com = nullptr;  // rate 1/2; must stay valid until `done` runs
    std::vector<u64> point;       // 2 n words (Ext2 point)
    gb_transcript t;              // the opening's transcript, its own preamble already absorbed
    u64* proof = nullptr;         // host, gb_basefold_proof_len(n, 1, q) words
    // called once, on the engine thread, after the proof is written (rc 0) or on failure
    std::function<void(int rc, const std::string& err)> done;
};

class OpenEngine;
// The engine for openings against `tab` (log_rate 1) with q queries on `device`; *rc is set
// to 0 or the error of starting it (then the returned engine is null).
OpenEngine* open_engine_create(const BfTable* tab, int q, int device, int* rc);
void open_engine_submit(OpenEngine* e, OpenTask&& task);
// Openings in flight or waiting (for tests and statistics).
size_t open_engine_in_flight(OpenEngine* e);
// Finishes every submitted opening, then stops the engine.
void open_engine_destroy(OpenEngine* e);

// The per-call path of the same tasks: each opening on the calling thread's stream
// (gb_basefold_open_ext2), then every commitment in coms is destroyed.  Synchronising.
int open_tasks_inline(void* table, int q, std::vector<OpenTask>& tasks, std::vector<void*>& coms);

}  // namespace gb
