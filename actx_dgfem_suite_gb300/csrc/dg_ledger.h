// Bookkeeping of the asynchronous operations a CTA has in flight on its
// mbarriers (bulk copies, tensor-core products), for kernels whose waits are
// bounded.
//
// Every thread keeps a ledger: the phase parity each barrier owes next (all
// threads wait on the barriers themselves), and, in the thread that issues
// the operations, which barriers still owe a completion.  A wait that gives
// up leaves its barrier owed at the same phase.  The kernels then leave
// their tile loop together (the decision is taken by __syncthreads_or over
// every thread's outcome, so it is uniform), and before the CTA releases its
// shared and tensor memory the issuing thread waits once more, bounded, for
// every completion it still owes.  Plain C++ so that the host can test it.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define DG_LEDGER_FN __host__ __device__ __forceinline__
#else
#define DG_LEDGER_FN inline
#endif

namespace dg {

template <int NBAR>
struct AsyncLedger {
  static_assert(NBAR >= 1 && NBAR <= 32, "one bit per barrier");
  uint32_t phase[NBAR];  // parity of the next completion of each barrier
  uint32_t owed;         // bit b: an operation issued on barrier b is not seen complete

  DG_LEDGER_FN void init() {
    for (int b = 0; b < NBAR; ++b) phase[b] = 0u;
    owed = 0u;
  }
  // the calling thread issued an operation that completes barrier b
  DG_LEDGER_FN void issue(int b) { owed |= 1u << b; }
  // outcome of a bounded wait for barrier b's next completion; returns `ok`
  DG_LEDGER_FN bool complete(int b, bool ok) {
    if (ok) {
      owed &= ~(1u << b);
      phase[b] ^= 1u;
    }
    return ok;
  }
  DG_LEDGER_FN bool owes(int b) const { return ((owed >> b) & 1u) != 0u; }
  DG_LEDGER_FN bool owes_any() const { return owed != 0u; }
};

}  // namespace dg
