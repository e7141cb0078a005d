// Packed trajectory batches: one persistent kernel runs many trajectories of
// mixed qubit counts, each CTA taking whole trajectories from a queue.
//
// The reference runs trajectories one after another
// (QuantumTrajectorySimulator::RunBatch, lib/qtrajectory.h:141-236); each
// fused gate, Norm, Multiply and ExpectationValue is a launch with host
// synchronisations in between (lib/qtrajectory.h:331-380).  Here the host
// compiles each trajectory into a short program of device ops (the Kraus
// choices that the lower probability bounds decide are already made; the
// others stay as CHANNEL ops whose choice is made on the device), and one
// launch runs the whole batch.  Shared by batch.cu and the host engine.
#pragma once

#include <cstdint>
#include <vector>

#include "traj_dev.h"

namespace qsg {

// Largest fused gate (targets) and the most controls a packed op may carry.
constexpr unsigned kBatchMaxK = 4;
constexpr unsigned kBatchMaxControls = 8;

enum BatchOpKind : uint32_t {
  kBatchSetZero = 0,   // |0..0>
  kBatchGate = 1,      // matrix on targets, optionally controlled
  kBatchChannel = 2,   // device-side Kraus choice (non-unitary channel)
  kBatchNormalize = 3  // state *= (float)(1 / sqrt(norm))
};

// One op of a trajectory program (64 bytes).
struct BatchOp {
  uint32_t kind;
  uint32_t geom;     // gate / channel: entry of the tile-geometry table
                     // (filled by batch_plan_geometries)
  uint64_t tmask;    // gate: target qubits (ascending = matrix bit order);
                     // channel: the channel's qubits
  uint64_t cmask;    // gate: control qubits
  uint64_t cvals;    // gate: control values at the control positions
  const float* mat;  // gate: row-major interleaved complex 2^k x 2^k
  const TrajChannelDev* ch;  // channel: the channel's device description
  double r;          // channel: the trajectory's draw for this op
  double cp0;        // channel: sum of the lower-bound probabilities
};
static_assert(sizeof(BatchOp) == 64, "BatchOp layout");

// Plans the shared-memory tile geometry of every GATE and CHANNEL op of the
// items (one table entry per distinct (n, targets, controls, values)),
// writes the entry index into each op and returns the table as bytes to
// upload.  Host code in batch.cu.
struct BatchItemDev;
int batch_plan_geometries(const BatchItemDev* items, size_t num_items,
                          BatchOp* ops, std::vector<unsigned char>* table);

// One trajectory of the batch.
struct BatchItemDev {
  uint64_t op_begin;   // index of its first op in the op array
  uint32_t num_ops;
  uint32_t n;          // qubits
  float* state;        // where it runs (null: the CTA's slot buffer)
  uint32_t log_begin;  // first entry of its device-choice log
  uint32_t pad;
};

// Launch shape and the run-time record of a packed batch.
struct BatchLaunch {
  unsigned ctas;          // persistent CTAs (a multiple of the SM count)
  unsigned threads;       // threads per CTA (128)
  float* slots;           // ctas x slot_floats (may be null if every item
  uint64_t slot_floats;   // has its own state buffer)
  const void* geoms;      // tile-geometry table (device)
  unsigned tile_kib;      // tile buffers per CTA: 32, 64 or 96 KiB
};

// Enqueues the persistent kernel on `stream`.  `counter` (one uint32 in
// device memory) must be zero; `log` receives one entry per CHANNEL op (the
// chosen Kraus index, 0xffffffff when none is chosen); `times` two
// %globaltimer readings (ns) per item; `error` is set nonzero on a bad op.
int batch_launch(void* stream, const BatchLaunch& l, const BatchItemDev* items,
                 uint32_t num_items, const BatchOp* ops, uint32_t* log,
                 unsigned long long* times, uint32_t* counter, int* error);

// Most CTAs of `threads` threads per SM the kernel can keep resident with
// a tile budget of tile_kib KiB.
int batch_max_ctas_per_sm(unsigned threads, unsigned tile_kib, int* out);

}  // namespace qsg
