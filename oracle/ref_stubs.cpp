// Link stubs for the reference's slice-streaming ring buffer
// (rtm/snapshot_buffer.cpp), whose shipped source does not compile (it
// resizes a std::vector of std::atomic slots). WaveEquationSolver creates the
// buffer in configure_rtm() and hands it every captured slice; the stubs below
// model the shipped ring as the oracle harness uses it, with no reader:
// capacity rounded up to a power of two (snapshot_buffer.cpp:7-10), the
// first `capacity` enqueues succeed, after which the write slot is full, so
// an enqueue is dropped and frees that slot and the next one succeeds, in
// turn (snapshot_buffer.cpp:28-56). Frames are not serialised (nothing reads
// them). Every other member aborts if reached.
#include "rtm/snapshot_buffer.h"
#include <cstdio>
#include <cstdlib>

namespace seismic {
[[noreturn]] static void stub_abort(const char* what) {
    std::fprintf(stderr, "oracle: reference %s is not built (off-path slice streaming)\n", what);
    std::abort();
}
LockFreeSnapshotBuffer::LockFreeSnapshotBuffer(size_t capacity) {
    capacity_ = 1;
    while (capacity_ < capacity) capacity_ <<= 1;
    mask_ = capacity_ - 1;
    write_index_.store(0);
    read_index_.store(0);
    sequence_counter_.store(0);
    total_enqueued_.store(0);
    total_dropped_.store(0);
    total_read_.store(0);
}
LockFreeSnapshotBuffer::~LockFreeSnapshotBuffer() {}
bool LockFreeSnapshotBuffer::try_enqueue(const RTMEngine::CapturedSlice&) {
    const uint64_t k = sequence_counter_.fetch_add(1);  // attempts so far
    if (k < capacity_ || ((k - capacity_) & 1u)) {
        write_index_.fetch_add(1);
        total_enqueued_.fetch_add(1);
        return true;
    }
    total_dropped_.fetch_add(1);
    return false;
}
bool LockFreeSnapshotBuffer::try_dequeue(RTMEngine::CapturedSlice&) { stub_abort("try_dequeue"); }
void LockFreeSnapshotBuffer::serialize_slice(const RTMEngine::CapturedSlice&, std::vector<uint8_t>&) {
    stub_abort("serialize_slice");
}
}  // namespace seismic
