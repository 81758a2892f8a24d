// columns_engine.h — host-side state of the packed column engine (columns.cu), shared with the
// continuous-batching service (service.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <map>
#include <vector>
#include "../../include/obgc.h"
#include "negatives.cuh"

namespace obgc {

constexpr int COL_MAXC = 64;    // columns per pack

template <typename T>
struct ColSlot {
    int64_t cell_off;           // first cell of the column's block (state at cell_off*NT, kappa at cell_off)
    int32_t Nz, steps_left, steps_done, pulse_step, pulse_k, live;
    T dz, dt, PAR0, mu0, pulse_amount, temp, sal, pad;   // temp / sal: surface T and S (gas exchange)
};

struct ColPack {
    int32_t first, count, cells, pad;
};

}  // namespace obgc

struct obgc_columns {
    obgc_columns_desc desc;
    int V = -1, NT = 0;
    size_t ts = 4;                           // state element size
    int prec = OBGC_PREC_F32;
    int threads = 256, cap = 1024;
    int names[16];
    obgc::NegativesSpec neg;
    double w0A = 0, w0B = 0;
    void* state = nullptr;                   // arena: column at cell_off holds [NT][Nz] from cell_off * NT
    void* kappa = nullptr;                   // arena: Nz + 1 face diffusivities from cell_off
    std::vector<obgc::ColSlot<double>> slots;
    std::vector<int> free_slots;
    std::map<int64_t, int64_t> free_cells;   // offset -> length
    void* d_slots = nullptr;
    int32_t* d_pack_slots = nullptr;
    obgc::ColPack* d_packs = nullptr;
    // pinned staging of the slot and pack tables, double-buffered: a buffer is rewritten only after
    // the copies that read it two stagings ago have completed (its event)
    void* h_slots[2] = {nullptr, nullptr};
    int32_t* h_pack_slots[2] = {nullptr, nullptr};
    obgc::ColPack* h_packs[2] = {nullptr, nullptr};
    cudaEvent_t tables_ev[2] = {nullptr, nullptr};
    bool tables_used[2] = {false, false};
    int tb = 0;                              // buffer of the latest staging
    cudaStream_t last_stream = nullptr;      // stream of the last launch or copy
    bool pending = false;                    // work may still be queued on last_stream
    cudaStream_t capture_stream = nullptr;   // private stream the launch graphs are captured on
    cudaGraphExec_t graph = nullptr;         // cached launches of obgc_columns_run
    int64_t graph_key[5] = {0, 0, 0, 0, 0};  // packs, steps, steps per launch, threads, pack cells
};


namespace obgc {
namespace cols {

// Wait for everything queued by the engine (launches and copies read its staging buffers).
int drain(obgc_columns* e);
// Dynamic shared memory above 48 KiB must be opted into before a launch (and before a capture).
int prepare_launch(obgc_columns* e, int cap);
// Pack the unfinished columns and copy the slot and pack tables to the device on `st`.
// Returns the number of packs (0: nothing to do) or a negative status.
int stage_tables(obgc_columns* e, int cap, cudaStream_t st);
int launch_any(obgc_columns* e, int npacks, int max_steps, int threads, int cap, cudaStream_t st);
// Host mirror of the kernel's bookkeeping: every unfinished column took min(steps, left) steps.
void account_steps(obgc_columns* e, int steps);
// Host bookkeeping of a new column (slot + arena block); no device work.  Returns a status.
int reserve_column(obgc_columns* e, const obgc_column_spec* sp, int64_t* slot);
// Return a column's slot and arena block to the free lists (no device work).
void release_column(obgc_columns* e, int64_t slot);

}  // namespace cols
}  // namespace obgc
