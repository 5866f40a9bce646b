// Point-cache (PC2) streaming writer: the on-disk output of the reference
// add-on's bake and realtime cache (session_manager.py:4624-4733).  Each
// frame a kernel on the solver's stream turns one cloth's positions into
// object-local coordinates (world @ R^T + t of the inverse object matrix)
// into a per-slot device buffer; a copy stream moves it into one of two
// pinned host buffers while the solver already runs the next frame, and a
// writer thread appends finished samples to the file.  The file is written
// under a temporary name with a zero sample count and, on a committed
// close, gets its final header and is renamed into place, as the
// reference's realtime cache does.
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>

#include "xpbd_host.cuh"

namespace xg {

namespace {

// local = world @ R^T + t in float32, R and t from the inverse object matrix
// (xpbd_core.py:652-655).
__global__ void k_pc2_local(const float4* pos, int n, const float* m, float* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    for (int r = 0; r < 3; ++r) {
        const float* row = m + 4 * r;
        out[3 * i + r] = ((p.x * row[0] + p.y * row[1]) + p.z * row[2]) + row[3];
    }
}

struct Pc2Writer {
    std::string path, tmp;
    FILE* f = nullptr;
    int V = 0, vstart = 0, start_frame = 0, samples = 0;
    float* dev[2] = {nullptr, nullptr};
    float* host[2] = {nullptr, nullptr};
    float* mat = nullptr;  // 12 floats on the device
    cudaEvent_t staged[2] = {nullptr, nullptr}, ready[2] = {nullptr, nullptr};
    cudaStream_t copy = nullptr;
    bool pending[2] = {false, false};
    int slot = 0;
    std::thread worker;
    std::mutex m;
    std::condition_variable cv;
    std::deque<int> queue;
    bool stop = false, io_error = false;
};

bool write_header(FILE* f, int vertex_count, int start_frame, int samples) {
    unsigned char h[32];
    std::memcpy(h, "POINTCACHE2\0", 12);
    const int version = 1;
    const float start = (float)start_frame, rate = 1.0f;
    std::memcpy(h + 12, &version, 4);
    std::memcpy(h + 16, &vertex_count, 4);
    std::memcpy(h + 20, &start, 4);
    std::memcpy(h + 24, &rate, 4);
    std::memcpy(h + 28, &samples, 4);
    return std::fwrite(h, 1, 32, f) == 32;
}

void writer_loop(Pc2Writer* W) {
    for (;;) {
        int s = -1;
        {
            std::unique_lock<std::mutex> lk(W->m);
            W->cv.wait(lk, [&] { return W->stop || !W->queue.empty(); });
            if (W->queue.empty()) return;
            s = W->queue.front();
            W->queue.pop_front();
        }
        const bool ok = cudaEventSynchronize(W->ready[s]) == cudaSuccess &&
                        std::fwrite(W->host[s], sizeof(float), (size_t)3 * W->V, W->f) == (size_t)3 * W->V;
        {
            std::lock_guard<std::mutex> lk(W->m);
            if (ok)
                W->samples += 1;
            else
                W->io_error = true;
            W->pending[s] = false;
        }
        W->cv.notify_all();
    }
}

void release(Pc2Writer* W) {
    if (W->worker.joinable()) {
        {
            std::lock_guard<std::mutex> lk(W->m);
            W->stop = true;
        }
        W->cv.notify_all();
        W->worker.join();
    }
    for (int s = 0; s < 2; ++s) {
        if (W->dev[s]) cudaFree(W->dev[s]);
        if (W->host[s]) cudaFreeHost(W->host[s]);
        if (W->staged[s]) cudaEventDestroy(W->staged[s]);
        if (W->ready[s]) cudaEventDestroy(W->ready[s]);
    }
    if (W->mat) cudaFree(W->mat);
    if (W->copy) cudaStreamDestroy(W->copy);
    if (W->f) std::fclose(W->f);
    W->f = nullptr;
}

}  // namespace

namespace host {

void* pc2_open(Solver* S, int cloth, const char* path, int start_frame) {
    if (!S || !path || cloth >= S->K) {
        fail("invalid PC2 writer request");
        return nullptr;
    }
    const int k = cloth < 0 ? 0 : cloth;
    Pc2Writer* W = new Pc2Writer();
    W->path = path;
    W->tmp = W->path + ".realtime.tmp";
    W->V = cloth < 0 ? S->nV : S->hp[k].V;
    W->vstart = cloth < 0 ? 0 : S->hp[k].vstart;
    W->start_frame = start_frame;
    W->f = std::fopen(W->tmp.c_str(), "w+b");
    const size_t n = (size_t)std::max(W->V, 1) * 3;
    bool ok = W->f != nullptr && write_header(W->f, W->V, start_frame, 0) &&
              cuda_ok(cudaStreamCreateWithFlags(&W->copy, cudaStreamNonBlocking), "PC2 writer stream") &&
              cuda_ok(cudaMalloc(reinterpret_cast<void**>(&W->mat), sizeof(float) * 12), "PC2 writer");
    for (int s = 0; s < 2 && ok; ++s)
        ok = cuda_ok(cudaMalloc(reinterpret_cast<void**>(&W->dev[s]), sizeof(float) * n), "PC2 writer") &&
             cuda_ok(cudaMallocHost(reinterpret_cast<void**>(&W->host[s]), sizeof(float) * n), "PC2 writer") &&
             cuda_ok(cudaEventCreateWithFlags(&W->staged[s], cudaEventDisableTiming), "PC2 writer") &&
             cuda_ok(cudaEventCreateWithFlags(&W->ready[s], cudaEventDisableTiming), "PC2 writer");
    if (!ok) {
        if (!W->f) fail("cannot open PC2 cache file " + W->tmp);
        release(W);
        std::remove(W->tmp.c_str());
        delete W;
        return nullptr;
    }
    W->worker = std::thread(writer_loop, W);
    return W;
}

// One sample from the cloth's current positions; matrix16 is the inverse
// object matrix, row-major 4x4 (null: identity).
bool pc2_write(Solver* S, void* writer, const float* matrix16) {
    Pc2Writer* W = reinterpret_cast<Pc2Writer*>(writer);
    if (!S || !W) return fail("invalid PC2 writer request");
    float m[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
    if (matrix16) std::memcpy(m, matrix16, sizeof(m));
    const int s = W->slot;
    {
        std::unique_lock<std::mutex> lk(W->m);
        W->cv.wait(lk, [&] { return !W->pending[s]; });  // the slot's previous sample is on disk
        if (W->io_error) return fail("PC2 cache write failed: " + W->tmp);
        W->pending[s] = true;
    }
    const int b = 256;
    bool ok = cuda_ok(cudaMemcpyAsync(W->mat, m, sizeof(m), cudaMemcpyHostToDevice, S->stream), "PC2 sample");
    if (ok && W->V > 0) k_pc2_local<<<(W->V + b - 1) / b, b, 0, S->stream>>>(S->pos[0] + W->vstart, W->V, W->mat, W->dev[s]);
    ok = ok && cuda_ok(cudaGetLastError(), "PC2 sample") && cuda_ok(cudaEventRecord(W->staged[s], S->stream), "PC2 sample") &&
         cuda_ok(cudaStreamWaitEvent(W->copy, W->staged[s], 0), "PC2 sample") &&
         cuda_ok(cudaMemcpyAsync(W->host[s], W->dev[s], sizeof(float) * 3 * (size_t)W->V, cudaMemcpyDeviceToHost, W->copy),
                 "PC2 sample") &&
         cuda_ok(cudaEventRecord(W->ready[s], W->copy), "PC2 sample");
    // the matrix upload is pageable: it completes before cudaMemcpyAsync returns,
    // so the next sample may overwrite `m` at once
    {
        std::lock_guard<std::mutex> lk(W->m);
        if (ok)
            W->queue.push_back(s);
        else
            W->pending[s] = false;
    }
    W->cv.notify_all();
    W->slot ^= 1;
    return ok;
}

// Finish: wait for queued samples; commit writes the final header and moves
// the file into place, otherwise the temporary file is removed.  Returns the
// sample count (-1 on failure).
long long pc2_close(void* writer, bool commit) {
    Pc2Writer* W = reinterpret_cast<Pc2Writer*>(writer);
    if (!W) {
        fail("invalid PC2 writer request");
        return -1;
    }
    {
        std::unique_lock<std::mutex> lk(W->m);
        W->cv.wait(lk, [&] { return W->queue.empty() && !W->pending[0] && !W->pending[1]; });
    }
    const long long samples = W->samples;
    bool ok = !W->io_error;
    if (commit && ok && samples > 0) {
        ok = std::fseek(W->f, 0, SEEK_SET) == 0 && write_header(W->f, W->V, W->start_frame, (int)samples) && std::fflush(W->f) == 0;
        release(W);
        ok = ok && std::rename(W->tmp.c_str(), W->path.c_str()) == 0;
        if (!ok) {
            std::remove(W->tmp.c_str());
            fail("cannot finish PC2 cache file " + W->path);
        }
    } else {
        release(W);
        std::remove(W->tmp.c_str());
        if (!ok) fail("PC2 cache write failed: " + W->tmp);
    }
    delete W;
    return ok ? samples : -1;
}

}  // namespace host
}  // namespace xg
