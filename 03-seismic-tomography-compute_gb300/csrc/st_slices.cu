// RTM slice frames and the mmap slice ring: the reference's visualisation
// stream (RTMEngine::extract_slices -> LockFreeSnapshotBuffer::serialize_slice
// -> MmapSnapshotWriter, rtm/rtm_engine.cpp:59-168, rtm/snapshot_buffer.cpp,
// rtm/mmap_writer.cpp) with the capture on the GPU.
//
// Capture: per slice spec, one kernel writes the 128-byte frame header and
// a second gathers the forward, adjoint and image-condition slices as FP64
// into the frame payload while folding the payload checksum. The checksum
// s = rotl13(s ^ w_1 ... ) over the n payload words is linear over XOR: word
// j (0-based) ends up rotated by 13 (n - j) mod 32, so every thread rotates
// its words by their position, the block XOR-reduces, and one atomicXor per
// block folds the block into the header's checksum field (the header kernel
// runs first on the same stream and leaves the field 0).
//
// Stream: frames go to pinned host slots with cudaMemcpyAsync; a host
// function enqueued behind the copy marks the slot full, and a writer
// thread appends full slots to the mmap file in capture order.
#include "st_slices.cuh"

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace {

constexpr int64_t kFileMagic = 0x52544D534E4150LL;
constexpr uint64_t kFrameMagic = 0x534C494345303031ULL;
constexpr int64_t kFileHeader = 15 * 8;  // sizeof(MmapFileHeader), packed
constexpr int64_t kFrameHeader = 128;     // SLICE_HEADER_SIZE

// MmapFileHeader field offsets (mmap_writer.h:28-38).
enum : int64_t { H_MAGIC = 0, H_SIZE = 8, H_FILE = 16, H_COUNT = 24, H_WOFF = 32, H_RING = 40, H_CAP = 48 };

}  // namespace

struct st_mmap_writer {
    std::string path;
    int fd = -1;
    uint8_t* base = nullptr;
    int64_t max_bytes = 0;
    std::mutex mu;
    int64_t frames_written = 0, frames_dropped = 0, total_bytes = 0, cycles = 0;
    int64_t* field(int64_t off) { return reinterpret_cast<int64_t*>(base + off); }
};

namespace stg {
namespace {

// -------------------------------------------------------------- capture
struct SliceGeom {
    int axis;
    int64_t index;
    int64_t d0, d1;
};

// Resolves a spec (index < 0 -> the middle plane, extract_slices :66-75).
// Returns false for VOLUME (nothing captured, capture_single_slice :160).
bool resolve(const st_slice_spec& sp, int64_t nx, int64_t ny, int64_t nz, SliceGeom* g) {
    const int64_t n[3] = {nx, ny, nz};
    if (sp.axis < 0 || sp.axis > 2) return false;
    g->axis = sp.axis;
    g->index = sp.index < 0 ? n[sp.axis] / 2 : sp.index;
    g->d0 = sp.axis == 0 ? ny : nx;
    g->d1 = sp.axis == 2 ? ny : nz;
    return true;
}

int64_t frame_bytes(const SliceGeom& g) { return kFrameHeader + 3 * 8 * g.d0 * g.d1; }

struct FrameHeader {
    uint32_t w[32];
};

FrameHeader make_header(const SliceGeom& g, int64_t timestep, double timestamp) {
    uint8_t b[128] = {};
    const int64_t bytes = 8 * g.d0 * g.d1;
    auto put = [&](int off, const void* v, int n) { std::memcpy(b + off, v, n); };
    const int32_t ax = g.axis;
    const int64_t size = frame_bytes(g), o0 = kFrameHeader, o1 = kFrameHeader + bytes, o2 = kFrameHeader + 2 * bytes;
    const uint64_t zero = 0;
    put(0, &kFrameMagic, 8);
    put(8, &timestep, 8);
    put(16, &ax, 4);
    put(20, &g.index, 8);
    put(28, &g.d0, 8);
    put(36, &g.d1, 8);
    put(44, &size, 8);
    put(52, &o0, 8);
    put(60, &o1, 8);
    put(68, &o2, 8);
    put(76, &bytes, 8);
    put(84, &bytes, 8);
    put(92, &bytes, 8);
    put(100, &timestamp, 8);
    put(108, &zero, 8);  // sequence_id; checksum (116) and reserved (120) stay 0
    FrameHeader h;
    std::memcpy(h.w, b, 128);
    return h;
}

__global__ void frame_header_kernel(FrameHeader h, uint32_t* dst) { dst[threadIdx.x] = h.w[threadIdx.x]; }

__device__ inline double load_field(const void* p, int kind, const Layout& L, int64_t ix, int64_t iy, int64_t iz) {
    if (kind == ST_FIELD_DEVICE_FP32) return (double)static_cast<const float*>(p)[L.at(ix, iy, iz)];
    const int64_t nyh = L.ny + 2, nzh = L.nz + 2;
    return static_cast<const double*>(p)[((ix + 1) * nyh + (iy + 1)) * nzh + (iz + 1)];
}

__device__ inline uint32_t rotl(uint32_t v, unsigned r) { return r ? (v << r) | (v >> (32u - r)) : v; }

__device__ inline double load_snapshot(const void* p, int kind, const unsigned* amax, const Layout& L, int64_t ix,
                                       int64_t iy, int64_t iz) {
    const long long i = (ix * L.ny + iy) * L.nz + iz;
    float v;
    if (kind == SNAP_BF16) v = __bfloat162float(static_cast<const __nv_bfloat16*>(p)[i]);
    else if (kind == SNAP_FP16) v = __half2float(static_cast<const __half*>(p)[i]);
    else v = static_cast<const float*>(p)[i];
    return (double)(v * (__uint_as_float(*amax) / SNAP_QMAX));
}

// One thread per payload double: q = 0 forward, 1 adjoint, 2 image condition.
__global__ void __launch_bounds__(256) slice_payload_kernel(SliceSrc S, SliceGeom g, uint8_t* frame) {
    const int64_t n = g.d0 * g.d1;
    const int64_t total = 3 * n;
    const uint64_t nwords = 2ull * (uint64_t)total;
    double* out = reinterpret_cast<double*>(frame + kFrameHeader);
    uint32_t x = 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int q = (int)(k / n);
        const int64_t e = k - (int64_t)q * n;
        const int64_t i = e / g.d1, j = e - i * g.d1;
        double v = 0.0;
        if (q < 2) {
            int64_t ix, iy, iz;
            if (g.axis == 0) { ix = g.index; iy = i; iz = j; }
            else if (g.axis == 1) { ix = i; iy = g.index; iz = j; }
            else { ix = i; iy = j; iz = g.index; }
            const void* src = q == 0 ? S.fwd : S.adj;
            if (q == 0 && S.fwd_snap != SNAP_NONE) v = load_snapshot(src, S.fwd_snap, S.fwd_amax, S.L, ix, iy, iz);
            else if (src) v = load_field(src, S.field_kind, S.L, ix, iy, iz);
        } else if (S.ic) {
            // the reference indexes the image with the slice's 2-D index (rtm_engine.cpp:108,131,153)
            v = S.ic_kind == ST_IMAGE_FP32 ? (double)static_cast<const float*>(S.ic)[e]
                                           : static_cast<const double*>(S.ic)[e];
        }
        if (!isfinite(v)) v = 0.0;
        out[k] = v;
        const unsigned long long u = __double_as_longlong(v);
        const uint64_t j0 = 2ull * (uint64_t)k;
        x ^= rotl((uint32_t)u, (unsigned)((13ull * (nwords - j0)) & 31u)) ^
             rotl((uint32_t)(u >> 32), (unsigned)((13ull * (nwords - j0 - 1)) & 31u));
    }
    for (int o = 16; o > 0; o >>= 1) x ^= __shfl_xor_sync(0xffffffffu, x, o);
    __shared__ uint32_t part[8];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t ^= part[w];
        atomicXor(reinterpret_cast<unsigned*>(frame + 116), t);
    }
}

int launch_frame(const SliceSrc& S, const SliceGeom& g, int64_t timestep, double timestamp, uint8_t* frame,
                 cudaStream_t st) {
    frame_header_kernel<<<1, 32, 0, st>>>(make_header(g, timestep, timestamp), reinterpret_cast<uint32_t*>(frame));
    count_launch();
    ST_CUDA(cudaGetLastError());
    const int64_t total = 3 * g.d0 * g.d1;
    const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, 152LL * 8));
    slice_payload_kernel<<<blocks, 256, 0, st>>>(S, g, frame);
    count_launch();
    ST_CUDA(cudaGetLastError());
    return ST_OK;
}

int check_sources(int64_t nx, int64_t ny, int64_t nz, int field_kind, int ic_kind) {
    ST_CHECK(nx > 0 && ny > 0 && nz > 0, ST_ERR_ARG, "bad slice grid extents");
    ST_CHECK(field_kind == ST_FIELD_DEVICE_FP32 || field_kind == ST_FIELD_REFERENCE_FP64, ST_ERR_ARG,
             "bad field kind %d", field_kind);
    ST_CHECK(ic_kind == ST_IMAGE_FP32 || ic_kind == ST_IMAGE_FP64, ST_ERR_ARG, "bad image kind %d", ic_kind);
    return ST_OK;
}

int resolve_all(int64_t nx, int64_t ny, int64_t nz, const st_slice_spec* specs, int n_specs,
                std::vector<SliceGeom>* out) {
    ST_CHECK(n_specs >= 0 && (specs || n_specs == 0), ST_ERR_ARG, "bad slice specs");
    const int64_t n[3] = {nx, ny, nz};
    out->clear();
    for (int k = 0; k < n_specs; ++k) {
        SliceGeom g;
        if (!resolve(specs[k], nx, ny, nz, &g)) {
            ST_CHECK(specs[k].axis == ST_SLICE_VOLUME, ST_ERR_ARG, "bad slice axis %d", (int)specs[k].axis);
            continue;
        }
        ST_CHECK(g.index < n[g.axis], ST_ERR_ARG, "slice index %lld outside the grid", (long long)g.index);
        out->push_back(g);
    }
    return ST_OK;
}

double wall_seconds() {
    // capture_timestamp: high_resolution_clock since its epoch, in seconds (rtm_engine.cpp:162-164)
    return std::chrono::duration<double>(std::chrono::high_resolution_clock::now().time_since_epoch()).count();
}

// ---------------------------------------------------------- mmap writer
int writer_append(st_mmap_writer* w, const uint8_t* frame, int64_t size) {
    ST_CHECK(w && w->base && frame && size > 0, ST_ERR_ARG, "bad frame");
    const int64_t rec = size + 8;
    ST_CHECK(kFileHeader + rec <= w->max_bytes, ST_ERR_ARG, "frame of %lld bytes does not fit the %lld-byte ring",
             (long long)size, (long long)w->max_bytes);
    std::lock_guard<std::mutex> lk(w->mu);
    int64_t cur = __atomic_load_n(w->field(H_WOFF), __ATOMIC_ACQUIRE);
    if (cur + rec > w->max_bytes) {  // reset_write_pointer (mmap_writer.cpp:178-183)
        __atomic_store_n(w->field(H_WOFF), kFileHeader, __ATOMIC_RELEASE);
        __atomic_fetch_add(w->field(H_RING), 1, __ATOMIC_ACQ_REL);
        ++w->cycles;
        cur = kFileHeader;
    }
    std::memcpy(w->base + cur, &size, 8);
    std::memcpy(w->base + cur + 8, frame, (size_t)size);
    __atomic_store_n(w->field(H_WOFF), cur + rec, __ATOMIC_RELEASE);
    __atomic_add_fetch(w->field(H_COUNT), 1, __ATOMIC_ACQ_REL);
    ++w->frames_written;
    w->total_bytes += rec;
    return ST_OK;
}

struct MappedFile {
    int fd = -1;
    uint8_t* base = nullptr;
    int64_t size = 0;
    ~MappedFile() {
        if (base) munmap(base, (size_t)size);
        if (fd >= 0) close(fd);
    }
};

int map_readonly(const char* path, MappedFile* m) {
    ST_CHECK(path, ST_ERR_ARG, "null path");
    m->fd = open(path, O_RDONLY);
    ST_CHECK(m->fd >= 0, ST_ERR_ARG, "cannot open %s", path);
    struct stat sb;
    ST_CHECK(fstat(m->fd, &sb) == 0 && sb.st_size >= kFileHeader, ST_ERR_ARG, "%s is not a slice ring", path);
    m->size = sb.st_size;
    void* p = mmap(nullptr, (size_t)m->size, PROT_READ, MAP_PRIVATE, m->fd, 0);
    ST_CHECK(p != MAP_FAILED, ST_ERR_ARG, "cannot map %s", path);
    m->base = static_cast<uint8_t*>(p);
    int64_t magic;
    std::memcpy(&magic, m->base + H_MAGIC, 8);
    ST_CHECK(magic == kFileMagic, ST_ERR_ARG, "%s: bad magic", path);
    return ST_OK;
}

}  // namespace
}  // namespace stg

// ------------------------------------------------------------ slice stream
struct st_slice_stream {
    enum SlotState { EMPTY = 0, IN_FLIGHT = 1, FULL = 2 };
    struct Slot {
        st_slice_stream* owner = nullptr;
        uint8_t* host = nullptr;  // pinned
        uint8_t* dev = nullptr;
        int64_t bytes = 0;
        int state = EMPTY;
    };
    int device = 0;
    int64_t nx = 0, ny = 0, nz = 0;
    std::vector<stg::SliceGeom> geom;
    st_mmap_writer* writer = nullptr;
    std::vector<Slot> slots;
    uint64_t head = 0, tail = 0;  // next slot to fill / to write
    std::mutex mu;
    std::condition_variable cv;
    std::thread thread;
    bool stop = false;
    int write_error = 0;
    int64_t captured = 0, dropped = 0, written = 0, bytes_written = 0;

    static void CUDART_CB on_copied(void* p) {
        Slot* s = static_cast<Slot*>(p);
        st_slice_stream* ss = s->owner;
        {
            std::lock_guard<std::mutex> lk(ss->mu);
            s->state = FULL;
        }
        ss->cv.notify_all();
    }

    void drain() {
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            cv.wait(lk, [&] { return stop || (tail < head && slots[tail % slots.size()].state == FULL); });
            if (tail < head && slots[tail % slots.size()].state == FULL) {
                Slot& s = slots[tail % slots.size()];
                lk.unlock();
                const int rc = stg::writer_append(writer, s.host, s.bytes);
                lk.lock();
                if (rc != ST_OK) write_error = rc;
                else {
                    ++written;
                    bytes_written += s.bytes + 8;
                }
                s.state = EMPTY;
                ++tail;
                cv.notify_all();
                continue;
            }
            if (stop) return;
        }
    }
};

namespace stg {

// Enqueues one frame per spec of the stream (shared by the C entry point and
// the solver's RTM loop).
int slice_stream_capture(st_slice_stream* ss, const SliceSrc& S, int64_t timestep, cudaStream_t st) {
    const double ts = wall_seconds();
    for (const auto& g : ss->geom) {
        st_slice_stream::Slot* slot;
        {
            std::lock_guard<std::mutex> lk(ss->mu);
            slot = &ss->slots[ss->head % ss->slots.size()];
            if (slot->state != st_slice_stream::EMPTY) {  // try_enqueue on a busy slot: dropped
                ++ss->dropped;
                continue;
            }
            slot->state = st_slice_stream::IN_FLIGHT;
            slot->bytes = frame_bytes(g);
            ++ss->head;
            ++ss->captured;
        }
        int rc = launch_frame(S, g, timestep, ts, slot->dev, st);
        if (rc == ST_OK && cudaMemcpyAsync(slot->host, slot->dev, (size_t)slot->bytes, cudaMemcpyDeviceToHost, st) !=
                               cudaSuccess)
            rc = ST_ERR_CUDA;
        if (rc == ST_OK && cudaLaunchHostFunc(st, st_slice_stream::on_copied, slot) != cudaSuccess) rc = ST_ERR_CUDA;
        if (rc != ST_OK) {
            // hand the slot to the writer as a failed (empty) frame so the ring order holds
            {
                std::lock_guard<std::mutex> lk(ss->mu);
                slot->bytes = 0;
                slot->state = st_slice_stream::FULL;
            }
            ss->cv.notify_all();
            cudaGetLastError();
            ST_CHECK(false, rc, "slice capture at step %lld failed", (long long)timestep);
        }
    }
    return ST_OK;
}

void slice_stream_extents(const st_slice_stream* ss, int64_t* nx, int64_t* ny, int64_t* nz) {
    *nx = ss->nx;
    *ny = ss->ny;
    *nz = ss->nz;
}

}  // namespace stg

using namespace stg;

extern "C" {

int st_mmap_writer_open(const char* path, int64_t max_bytes, st_mmap_writer** out) {
    ST_CHECK(path && out, ST_ERR_ARG, "null argument");
    ST_CHECK(max_bytes > kFileHeader, ST_ERR_ARG, "ring of %lld bytes is smaller than its header",
             (long long)max_bytes);
    *out = nullptr;
    std::unique_ptr<st_mmap_writer> w(new st_mmap_writer());
    w->path = path;
    w->max_bytes = max_bytes;
    w->fd = open(path, O_RDWR | O_CREAT | O_TRUNC, 0644);
    ST_CHECK(w->fd >= 0, ST_ERR_ARG, "cannot create %s", path);
    if (ftruncate(w->fd, max_bytes) != 0) {
        close(w->fd);
        ST_CHECK(false, ST_ERR_ALLOC, "cannot size %s to %lld bytes", path, (long long)max_bytes);
    }
    void* p = mmap(nullptr, (size_t)max_bytes, PROT_READ | PROT_WRITE, MAP_SHARED, w->fd, 0);
    if (p == MAP_FAILED) {
        close(w->fd);
        ST_CHECK(false, ST_ERR_ALLOC, "cannot map %s", path);
    }
    w->base = static_cast<uint8_t*>(p);
    const int64_t hdr[15] = {kFileMagic, kFileHeader, max_bytes, 0, kFileHeader, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    std::memcpy(w->base, hdr, sizeof(hdr));
    w->cycles = 1;  // open counts one mapping cycle (mmap_writer.cpp:125)
    *out = w.release();
    return ST_OK;
}

int st_mmap_writer_write_frame(st_mmap_writer* w, const uint8_t* frame, int64_t size) {
    return writer_append(w, frame, size);
}

int st_mmap_writer_info(st_mmap_writer* w, int64_t out[7]) {
    ST_CHECK(w && out, ST_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> lk(w->mu);
    out[0] = *w->field(H_COUNT);
    out[1] = *w->field(H_WOFF);
    out[2] = w->max_bytes;
    out[3] = w->frames_written;
    out[4] = w->frames_dropped;
    out[5] = w->total_bytes;
    out[6] = w->cycles;
    return ST_OK;
}

int st_mmap_writer_close(st_mmap_writer* w) {
    if (!w) return ST_OK;
    if (w->base) {
        msync(w->base, (size_t)w->max_bytes, MS_SYNC);
        munmap(w->base, (size_t)w->max_bytes);
    }
    if (w->fd >= 0) close(w->fd);
    delete w;
    return ST_OK;
}

int st_mmap_read_frame(const char* path, int64_t index, uint8_t* out, int64_t cap, int64_t* size) {
    MappedFile m;
    ST_TRY(map_readonly(path, &m));
    int64_t end;
    std::memcpy(&end, m.base + H_WOFF, 8);
    end = std::min(end, m.size);
    int64_t off = kFileHeader;
    for (int64_t k = 0; off + 8 <= end; ++k) {
        int64_t n;
        std::memcpy(&n, m.base + off, 8);
        off += 8;
        ST_CHECK(n > 0 && off + n <= m.size, ST_ERR_ARG, "%s: corrupt record at %lld", path, (long long)(off - 8));
        if (k == index) {
            if (size) *size = n;
            if (out) {
                ST_CHECK(cap >= n, ST_ERR_ARG, "frame of %lld bytes exceeds the buffer", (long long)n);
                std::memcpy(out, m.base + off, (size_t)n);
            }
            return ST_OK;
        }
        off += n;
    }
    ST_CHECK(false, ST_ERR_ARG, "%s has no frame %lld", path, (long long)index);
}

int st_mmap_count_frames(const char* path, int64_t* count) {
    ST_CHECK(count, ST_ERR_ARG, "null argument");
    MappedFile m;
    ST_TRY(map_readonly(path, &m));
    std::memcpy(count, m.base + H_COUNT, 8);
    return ST_OK;
}

int64_t st_slice_frame_bytes(int64_t nx, int64_t ny, int64_t nz, const st_slice_spec* spec) {
    SliceGeom g;
    if (!spec || !resolve(*spec, nx, ny, nz, &g)) return 0;
    return frame_bytes(g);
}

int st_capture_slice_frames(int64_t nx, int64_t ny, int64_t nz, const st_slice_spec* specs, int n_specs,
                            const void* fwd, const void* adj, int field_kind, const void* ic, int ic_kind,
                            int64_t timestep, double timestamp, uint8_t* frames, int64_t cap, int64_t* bytes,
                            void* stream) {
    ST_TRY(check_sources(nx, ny, nz, field_kind, ic_kind));
    std::vector<SliceGeom> gs;
    ST_TRY(resolve_all(nx, ny, nz, specs, n_specs, &gs));
    int64_t total = 0;
    for (const auto& g : gs) total += frame_bytes(g);
    ST_CHECK(total <= cap && (frames || total == 0), ST_ERR_ARG, "frames need %lld bytes, %lld given",
             (long long)total, (long long)cap);
    ST_CHECK((reinterpret_cast<uintptr_t>(frames) & 7) == 0, ST_ERR_ARG, "frame buffer must be 8-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const SliceSrc S{fwd, adj, ic, field_kind, ic_kind, make_layout(nx, ny, nz)};
    int64_t o = 0;
    for (const auto& g : gs) {
        ST_TRY(launch_frame(S, g, timestep, timestamp, frames + o, st));
        o += frame_bytes(g);
    }
    if (bytes) *bytes = total;
    return ST_OK;
}

int st_slice_stream_create(const char* path, int64_t max_bytes, int64_t nx, int64_t ny, int64_t nz,
                           const st_slice_spec* specs, int n_specs, int capacity, int device,
                           st_slice_stream** out) {
    ST_CHECK(out, ST_ERR_ARG, "null argument");
    *out = nullptr;
    ST_CHECK(capacity > 0 && capacity <= 4096, ST_ERR_ARG, "slot capacity must be in [1, 4096]");
    ST_CHECK(nx > 0 && ny > 0 && nz > 0, ST_ERR_ARG, "bad slice grid extents");
    std::unique_ptr<st_slice_stream> ss(new st_slice_stream());
    ST_TRY(resolve_all(nx, ny, nz, specs, n_specs, &ss->geom));
    ss->device = device;
    ss->nx = nx;
    ss->ny = ny;
    ss->nz = nz;
    int64_t most = 0;
    for (const auto& g : ss->geom) {
        most = std::max(most, frame_bytes(g));
        ST_CHECK(kFileHeader + frame_bytes(g) + 8 <= max_bytes, ST_ERR_ARG, "a %lld-byte frame does not fit the ring",
                 (long long)frame_bytes(g));
    }
    ST_CUDA(cudaSetDevice(device));
    // the reference's ring holds up to `capacity` frames of any size; here
    // each slot is a pinned frame-sized buffer, so the slot count is capped
    // at 256 MB of pinned memory
    if (most > 0) capacity = (int)std::max<int64_t>(1, std::min<int64_t>(capacity, (256ll << 20) / most));
    ss->slots.resize((size_t)capacity);
    for (auto& s : ss->slots) {
        s.owner = ss.get();
        if (most > 0) {
            if (cudaMallocHost(&s.host, (size_t)most) != cudaSuccess || cudaMalloc(&s.dev, (size_t)most) != cudaSuccess) {
                cudaGetLastError();
                for (auto& t : ss->slots) {
                    cudaFreeHost(t.host);
                    cudaFree(t.dev);
                }
                ST_CHECK(false, ST_ERR_ALLOC, "slice stream slots of %lld bytes", (long long)most);
            }
        }
    }
    int rc = st_mmap_writer_open(path, max_bytes, &ss->writer);
    if (rc != ST_OK) {
        for (auto& t : ss->slots) {
            cudaFreeHost(t.host);
            cudaFree(t.dev);
        }
        return rc;
    }
    st_slice_stream* raw = ss.get();
    ss->thread = std::thread([raw] { raw->drain(); });
    *out = ss.release();
    return ST_OK;
}

int st_slice_stream_capture(st_slice_stream* ss, const void* fwd, const void* adj, int field_kind, const void* ic,
                            int ic_kind, int64_t timestep, void* stream) {
    ST_CHECK(ss, ST_ERR_ARG, "null argument");
    ST_TRY(check_sources(ss->nx, ss->ny, ss->nz, field_kind, ic_kind));
    ST_CUDA(cudaSetDevice(ss->device));
    const SliceSrc S{fwd, adj, ic, field_kind, ic_kind, make_layout(ss->nx, ss->ny, ss->nz)};
    return slice_stream_capture(ss, S, timestep, static_cast<cudaStream_t>(stream));
}

int st_slice_stream_flush(st_slice_stream* ss) {
    ST_CHECK(ss, ST_ERR_ARG, "null argument");
    std::unique_lock<std::mutex> lk(ss->mu);
    const bool done = ss->cv.wait_for(lk, std::chrono::seconds(120), [&] { return ss->tail == ss->head; });
    ST_CHECK(done, ST_ERR_TIMEOUT, "slice stream: %llu frames still in flight after 120 s",
             (unsigned long long)(ss->head - ss->tail));
    ST_CHECK(ss->write_error == 0, ss->write_error, "slice stream: a frame could not be written");
    return ST_OK;
}

int st_slice_stream_stats(st_slice_stream* ss, int64_t out[4]) {
    ST_CHECK(ss && out, ST_ERR_ARG, "null argument");
    std::lock_guard<std::mutex> lk(ss->mu);
    out[0] = ss->captured;
    out[1] = ss->dropped;
    out[2] = ss->written;
    out[3] = ss->bytes_written;
    return ST_OK;
}

int st_slice_stream_destroy(st_slice_stream* ss) {
    if (!ss) return ST_OK;
    const int rc = st_slice_stream_flush(ss);
    {
        std::lock_guard<std::mutex> lk(ss->mu);
        ss->stop = true;
    }
    ss->cv.notify_all();
    if (rc == ST_OK && ss->thread.joinable()) ss->thread.join();
    if (rc != ST_OK) {
        // frames still in flight would touch the slots: keep them (and the thread) alive
        if (ss->thread.joinable()) ss->thread.detach();
        return rc;
    }
    st_mmap_writer_close(ss->writer);
    cudaSetDevice(ss->device);
    for (auto& t : ss->slots) {
        cudaFreeHost(t.host);
        cudaFree(t.dev);
    }
    delete ss;
    return ST_OK;
}

}  // extern "C"
