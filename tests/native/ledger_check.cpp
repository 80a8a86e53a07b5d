// Host check of the asynchronous-operation ledger the tcgen05 kernels use to
// leave their tile loop after a bounded wait gives up (dg_ledger.h).  Each
// scenario replays the sequence of issues and wait outcomes one thread sees
// and checks which completions it still owes, and at which phase.
#include <cstdio>
#include <cstdlib>

#include "../../actx_dgfem_suite_gb300/csrc/dg_ledger.h"

static int failures = 0;
#define CHECK(cond)                                                  \
  do {                                                               \
    if (!(cond)) {                                                   \
      std::printf("FAIL line %d: %s\n", __LINE__, #cond);            \
      ++failures;                                                    \
    }                                                                \
  } while (0)

int main() {
  constexpr int kMma = 0, kIn0 = 1;
  {  // a full tile loop with every wait completing: nothing is owed at the end
    dg::AsyncLedger<3> led;
    led.init();
    led.issue(kIn0);                      // prefetch of tile 0
    for (int tile = 0; tile < 5; ++tile) {
      const int b = tile & 1;
      if (tile + 1 < 5) led.issue(kIn0 + (b ^ 1));  // prefetch of the next tile
      CHECK(led.complete(kIn0 + b, true));
      for (int c = 0; c < 2; ++c) {       // volume and LIFT products
        led.issue(kMma);
        CHECK(led.complete(kMma, true));
      }
    }
    CHECK(!led.owes_any());
    CHECK(led.phase[kMma] == 0u);         // 10 completions: parity back to 0
    CHECK(led.phase[kIn0] == 1u && led.phase[kIn0 + 1] == 0u);
  }
  {  // products that never complete: owed at the phase that was waited for
    dg::AsyncLedger<3> led;
    led.init();
    led.issue(kMma);
    CHECK(led.complete(kMma, true));
    led.issue(kMma);
    CHECK(!led.complete(kMma, false));
    CHECK(led.owes(kMma));
    CHECK(led.phase[kMma] == 1u);          // still the phase of the second commit
    CHECK(!led.owes(kIn0) && !led.owes(kIn0 + 1));
  }
  {  // an input copy that never arrives while the next tile's copy is in flight
    dg::AsyncLedger<3> led;
    led.init();
    led.issue(kIn0);                       // tile 0 into buffer 0
    led.issue(kIn0 + 1);                   // tile 1 into buffer 1
    CHECK(!led.complete(kIn0, false));
    CHECK(led.owes(kIn0) && led.owes(kIn0 + 1) && !led.owes(kMma));
    CHECK(led.phase[kIn0] == 0u && led.phase[kIn0 + 1] == 0u);
  }
  {  // a thread that only waits never owes anything, whatever the outcome
    dg::AsyncLedger<1> led;
    led.init();
    CHECK(led.complete(0, true));
    CHECK(!led.complete(0, false));
    CHECK(!led.owes_any());
    CHECK(led.phase[0] == 1u);
  }
  if (failures) return EXIT_FAILURE;
  std::printf("ledger ok\n");
  return EXIT_SUCCESS;
}
