// eager.cuh - eager (per-batch) executors.
#pragma once
#include "runtime.h"

namespace sjbg {
struct EagerState {
    int placeholder = 0;
};
int eager_init(sjbg_handle *h);
}  // namespace sjbg
