// cp3_trace.hpp -- NVTX ranges in the "cudaprob3_gb300" domain around the library's host-side
// work: a propagator's compute and result transfers, a batch's configure / tune / run, and
// each launch the serving loop packs.  NVTX v3 is header-only: without a tool attached
// (Nsight Systems, `ncu --nvtx`) a range costs a pointer test; with one, the ranges name what
// the kernels in them belong to, e.g.
//   ncu --nvtx --nvtx-include "cudaprob3_gb300@batch_run/" ...
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace cp3 {

inline nvtxDomainHandle_t trace_domain() {
    static const nvtxDomainHandle_t d = nvtxDomainCreateA("cudaprob3_gb300");
    return d;
}

// A range open for the lifetime of the object.
class TraceRange {
  public:
    explicit TraceRange(const char* name) {
        nvtxEventAttributes_t a{};
        a.version = NVTX_VERSION;
        a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
        a.messageType = NVTX_MESSAGE_TYPE_ASCII;
        a.message.ascii = name;
        nvtxDomainRangePushEx(trace_domain(), &a);
    }
    ~TraceRange() { nvtxDomainRangePop(trace_domain()); }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace cp3
