// Device-resident SparseTensor4d: the m kept nonzeros of a compressed T2 in
// the reference's slot order (include/sparse_tensor.hpp:13-100), plus the
// bucketed (CSR) views the contraction kernels read.
#pragma once
#include "common.cuh"

// One bucketing of the nonzeros by an ordered pair of index slots (pa, pb):
// bucket P = slot[pa] * dims[pb] + slot[pb].  order[] lists the nonzero slots
// of bucket P in ascending slot order between bptr[P] and bptr[P+1].
struct Bucketing {
  int pa = -1, pb = -1;
  int64_t nbuckets = 0;
  int* bptr = nullptr;       // [nbuckets + 1]
  unsigned* order = nullptr; // [m]
  bool valid = false;        // false after a re-compression: rebuilt in place on next use
};

struct FriccSparse {
  int64_t dims[4] = {0, 0, 0, 0};
  int64_t m = 0;            // kept nonzeros
  int64_t n_largest = 0;    // |D|: entries kept exactly (compression "fri"), valid when !pending
  // Written by the device at the end of an asynchronous compression and read
  // back at the next blocking call on the handle: [0] |D|, [1] error bits.
  unsigned long long* meta = nullptr;
  bool pending = false;     // the status lives in meta (asynchronous compressions)
  int status = 0;           // status of the last compression once read back
  int64_t* flat = nullptr;  // [m] flat C-order index into the dense tensor
  double* vals = nullptr;   // [m]
  int* slots = nullptr;     // [m][4] unpacked (i, j, a, b)
  Bucketing buck[6];
  cudaStream_t owner_stream = nullptr;
  int device = 0;
};

// Index of the cached bucketing for (pa, pb), building it on first use.
int fricc_sparse_bucketing(FriccSparse* T, int pa, int pb, cudaStream_t st, Bucketing** out);

// R compressed tensors of one shape (a replica batch), stacked: replica r's
// arrays start r*m entries (flat, vals, slots: r*4*m ints) after the base.
// which = 0: the compression the T2 terms use, 1: the one the W
// intermediates use (the two compressions of an iteration).
struct BatchBucketing {
  int pa = -1, pb = -1;
  int64_t nbuckets = 0;
  int* bptr = nullptr;        // [R][nbuckets + 1]
  unsigned* order = nullptr;  // [R][m]
  bool valid = false;
};

struct FriccSparseBatch {
  int R = 0;
  int64_t dims[4] = {0, 0, 0, 0};
  int64_t m = 0;
  int64_t* flat[2] = {nullptr, nullptr};              // [R][m]
  double* vals[2] = {nullptr, nullptr};               // [R][m]
  int* slots[2] = {nullptr, nullptr};                 // [R][m][4]
  unsigned long long* meta[2] = {nullptr, nullptr};   // [R][2]: |D|, error bits
  BatchBucketing buck[2][6];
  bool compressed = false;
  cudaStream_t owner_stream = nullptr;
  int device = 0;
};

int fricc_batch_bucketing(FriccSparseBatch* B, int which, int pa, int pb, cudaStream_t st, BatchBucketing** out);
