// Internal structures of the GB300 segregated solid solver library.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "s4g.h"

namespace s4g {

// Host-side result of the once-per-mesh preparation (renumbering, DIC
// scheduling parts, CSR in the storage order).  All indices are storage
// indices unless named otherwise.
struct HostPrep {
  int nC = 0, nI = 0, nB = 0, nParts = 0;
  std::vector<int> s2c;        // storage row -> caller cell
  std::vector<int> c2s;        // caller cell -> storage row
  std::vector<int> solverRank; // storage row -> position in the DIC (solver) order

  // cell-to-cell CSR over internal faces, lower entries first, each part
  // sorted by solver rank of the neighbour
  std::vector<int> rowptr, col, fidx;  // fidx: face index, ~face if the row is the neighbour side
  // internal faces in storage orientation (owner = lower storage row)
  std::vector<int> fown, fnei;
  std::vector<int> fcaller;            // caller face index
  std::vector<char> fflip;             // orientation flipped w.r.t. the caller
  // boundary faces sorted by storage cell
  std::vector<int> bcell, bpatch, bcaller, browptr;

  // DIC scheduling: parts are contiguous storage ranges; local levels inside
  std::vector<int> partStart;          // [nParts+1]
  std::vector<int> lvlOff;             // [nParts+1] offsets into lvlStart
  std::vector<int> lvlStart;           // row offsets of local levels (absolute), per part nl+1 entries
  std::vector<int> upPtr, upIdx;       // upstream parts (forward sweep deps)
  std::vector<int> dnPtr, dnIdx;       // downstream parts (backward sweep deps)
  int partDepth = 0, maxLocalLevels = 0, globalLevels = 0;
  // shared-memory staging of the sweeps: remote rows each part reads
  // (forward: lower neighbours in earlier parts; backward: upper neighbours
  // in later parts) and, per CSR entry, the shared-memory slot of its
  // column: local row index, maxRows + halo index, or the zero slot for an
  // entry a subdomain DIC ignores.  Lower entries >= 0, upper entries ~slot.
  std::vector<int> haloFPtr, haloFIdx, haloBPtr, haloBIdx, slot;
  std::vector<int> lowCnt;  // per row: number of lower entries (they come first)
  int maxRows = 0, maxHalo = 0, maxEntries = 0;

  // Processor-local DIC (subdomain runs only): per part, the in-part
  // entries of each row, lower entries in CSR order then upper entries in
  // reverse CSR order, as (CSR entry, local row) pairs.  Each part's range
  // is padded to a multiple of 8 entries (padding: locSrc -1, locIdx 0) so
  // that it can be staged with 16-byte copies.  locMeta per row, padded to a
  // multiple of 4 per part: entry offset within the part (bits 0-15), lower
  // count (16-23), upper count (24-31).
  std::vector<int> locEntStart, locSrc, locMetaStart;
  std::vector<uint16_t> locIdx;
  std::vector<uint32_t> locMeta;
  // per part, for one 32-byte load: {partStart, rows, locEntStart, entries}
  // and {locMetaStart, metas, lvlOff, levels}
  std::vector<int> locDesc;  // [nParts][8]
  int maxLocEntries = 0, maxLocMeta = 0;
  // fixed-slot tables (every row has 3 lower then 3 upper slots, padded
  // with a zero coefficient on the zero row maxRows): locSrc/locIdx hold
  // the slots, locMeta is empty
  bool locSlots = false;
};

// Sets the calling thread's s4g_last_error message (the server reports a
// worker's error to the thread that polls).
void setLastError(const std::string& msg);

// Builds the preparation.  Returns S4G_OK or S4G_BAD_ARG with `err` set.
s4g_status prepareMesh(const s4g_mesh_desc* d, const s4g_mesh_opts* o,
                       HostPrep& hp, std::string& err);

}  // namespace s4g
