// stream.cuh - event-time streaming loop.
#pragma once
#include "runtime.h"

namespace sjbg {
struct StreamState {
    int placeholder = 0;
};
}  // namespace sjbg
