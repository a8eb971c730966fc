// Link stubs for the reference's slice-streaming ring buffer
// (rtm/snapshot_buffer.cpp), whose shipped source does not compile (it
// resizes a std::vector of std::atomic slots). WaveEquationSolver only
// touches the buffer after configure_rtm() enables RTM streaming, which the
// oracle harness never calls; every stub aborts if reached.
#include "rtm/snapshot_buffer.h"
#include <cstdio>
#include <cstdlib>

namespace seismic {
[[noreturn]] static void stub_abort(const char* what) {
    std::fprintf(stderr, "oracle: reference %s is not built (off-path slice streaming)\n", what);
    std::abort();
}
LockFreeSnapshotBuffer::LockFreeSnapshotBuffer(size_t) { stub_abort("LockFreeSnapshotBuffer"); }
LockFreeSnapshotBuffer::~LockFreeSnapshotBuffer() {}
bool LockFreeSnapshotBuffer::try_enqueue(const RTMEngine::CapturedSlice&) { stub_abort("try_enqueue"); }
bool LockFreeSnapshotBuffer::try_dequeue(RTMEngine::CapturedSlice&) { stub_abort("try_dequeue"); }
void LockFreeSnapshotBuffer::serialize_slice(const RTMEngine::CapturedSlice&, std::vector<uint8_t>&) {
    stub_abort("serialize_slice");
}
}  // namespace seismic
