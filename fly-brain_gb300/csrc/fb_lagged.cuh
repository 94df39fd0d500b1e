// The delay-scheduled single-brain step kernel (fb_lagged.cu): arguments and launch glue.
#pragma once
#include <vector>

#include "fb_internal.cuh"

namespace fb {

constexpr int kLagRing = 64;  // ring depth of the per-step counters and lists (a power of two)
constexpr int kLagThreads = 1024;  // threads per block
constexpr int kLagPer = 2;        // neurons per thread at most (tile and driven blocks)
constexpr int kLagTileWorkers = kLagThreads - 64;  // tile-block threads that update neurons
constexpr int kLagHelpMax = 32;   // driven spikes of one step a tile block pushes at most
constexpr int kLagMaxDB = 2;      // driven blocks at most (each owns a contiguous part of the list)
constexpr int kLagSplit = 512;    // driven lists at least this long are split over two blocks
// The tile blocks push the driven block's spikes `help` steps late (their helper warp lists a
// step's share one step before the workers push it). The driven block releases its spike lists
// every help - 1 steps (the release holds up its warp about as long as the rest of a step): with a
// delay of at least 8 steps help = 4, from kLagPairDelay steps 3, otherwise 2. The lag bound is
// L = D - help >= 2 (a block's own completion of step s - 1 is published at step s, before it
// checks the lag of step s + 1).
constexpr int kLagPairDelay = 6;
inline int lag_help(int D) { return D >= 8 ? 4 : D >= kLagPairDelay ? 3 : 2; }

struct LagArgs {
  Trial *G;  // the brain's device header: scalars are written back at the end
  int32_t N;
  int64_t E;
  int32_t T;      // steps of this launch
  int32_t D;      // arrival delay in steps (nslots - 1)
  int32_t S;      // arrival slots of the contribution buffer (2 D)
  int32_t L;      // lag bound D - help
  int32_t help;   // steps after which the tile blocks push the driven block's spikes
  int32_t dbPub;  // steps per release of the driven block's spike lists (help - 1)
  int32_t nTB;    // tile blocks (grid - nDB)
  int32_t cap;    // neurons per tile block (capacity)
  int32_t nD;     // driven-list length
  int32_t nDcap;  // capacity of one driven block (>= its part of the list)
  int32_t nDall;  // capacity of a step's driven spike list (>= nD)
  int32_t nDB;    // driven blocks: block d owns the list's entries dLo[d] .. dLo[d + 1] - 1
  int32_t dLo[kLagMaxDB + 1];
  int32_t hasBg, bgCap;
  // header constants (lif.c's f32 header)
  float dt, vRest, vThresh, vReset, tRef, adaptInc, depU, dE, dTr, dA, kRec, kM, dtS;
  float eExc, eInh, cE, cI, bgEvents, bgAmp;
  int32_t coba, pad0;
  // graph
  const uint32_t *indptr, *indices;
  const float *W, *sign;
  const uint32_t *inOff;  // [N+1] in-degree prefix: target q's bucket entries start at inOff[q]
  const uint4 *edgeRec;   // [E] per edge: target's count slot, its first bucket entry, their end
  // state
  float *v, *gE, *gI, *refr, *trace, *adapt, *res, *bias, *thr, *drive;
  uint32_t *spikeCount;
  int32_t *ring, *ringCount;
  const int32_t *driven;
  // ownership
  const int32_t *ndIds;        // non-driven neuron ids, ascending
  const int32_t *ndLo;         // [nTB + 1] first ndIds entry of each tile block
  const int32_t *drvPosOf;     // [N] place of each neuron in the driven list, -1 if not driven
  // contribution buckets: counts [S][cntStride] (neuron ids, then the driven list's own slots
  // N + position), entries [S][E] ({(rank << 1) | inh, f32 bits})
  int64_t cntStride;
  uint32_t *cnt;
  uint2 *buf;
  uint32_t *pend0;  // [N] in-flight arrival marks at launch
  // synchronisation and per-step lists (rings of kLagRing steps)
  uint32_t *done;     // completion counters
  uint32_t *dbDone;   // [nDB] steps whose spike lists each driven block has released
  // [kLagRing][kLagMaxDB] ((step + 1) << 32) | the driven block's entries not refractory at the
  // step (its share of the step's draws), one word so that no fence is needed
  unsigned long long *liveTag;
  uint32_t *bgReady;  // steps whose background targets are published
  uint32_t *bgList;   // [kLagRing][bgCap]
  int32_t *bgCount;   // [kLagRing]
  uint4 *dbList;      // [kLagRing][nDall][2] driven spikes, driven block d's from entry dLo[d],
                      // any order: {id, rank key, amplitude bits, 0}, {row start, row end, 0, 0}
  int32_t *dbCnt;     // [kLagRing][nDB] spikes of the step, by driven block
  int32_t *tStage;    // [kLagRing][nTB][cap] tile spikes (local indices, ascending)
  int32_t *tCnt;      // [kLagRing][nTB]
  // per-step log (launches of at most kLagRing steps)
  int32_t log, pad1;
  int32_t *logCount, *logRaster;
  int64_t logCap, logRasterCap;
  int32_t *stepTot;  // [kLagRing] fired count per step (logging)
  unsigned long long *prof;  // optional phase accumulators (null: off)
  const uint32_t *jumpHex;   // lagged_jump_tables()
  uint32_t *barCount;
  int32_t *err;
  int64_t timeoutNs;
  int32_t tripStep;  // test hook: the first tile block waits at this step on a flag nothing sets (-1: off)
  int32_t pad;
};

// Jump tables of the driven block: M^(v 16^i) (i < 3, v = 1..15), M^4096, and M^l (l < 32, by lane).
void lagged_jump_tables(std::vector<uint32_t> &tab);
cudaError_t launch_edge_records(const uint32_t *indices, const uint8_t *dup, const uint32_t *inOff,
                                const int32_t *posOf, int32_t N, int64_t E, uint4 *out, cudaStream_t st);
size_t lagged_smem_bytes(int cap, int nDcap, int nDall);
int lagged_blocks_per_sm(size_t smem);
cudaError_t launch_lagged(const LagArgs &a, int grid, size_t smem, cudaStream_t st);

}  // namespace fb
