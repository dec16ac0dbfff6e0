// snapshot.cu -- the reference's raw snapshot format (src/simulation_io.c:16-149:
// the slab, N*SIM_DOF reals, written and read as one block with no header)
// for resident simulations, without a host sync per snapshot.
//
// sfgpu_save_raw queues a device-to-host copy of the slab into one of two
// page-locked staging buffers on the simulation's stream, followed by a host
// callback that hands the buffer to a writer thread; the caller's stream
// goes on with the next steps while the file is written.  A third snapshot
// issued while both buffers are still being written waits for one of them.
// sfgpu_snapshot_wait blocks until every queued snapshot is on disk and
// returns the first write error.  sfgpu_read_raw reads a file into staging
// memory and uploads it (synchronous).
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>

#include "internal.cuh"

namespace {

constexpr int SNAP_BUFFERS = 2;

struct SnapJob {
    int buf;
    std::string path;
};

}  // namespace

struct SnapshotWriter {
    size_t bytes = 0;
    float* staging[SNAP_BUFFERS] = {nullptr, nullptr};
    bool busy[SNAP_BUFFERS] = {false, false};
    std::mutex mu;
    std::condition_variable cv;
    std::deque<SnapJob> ready;   // copies landed, waiting for the writer
    int queued = 0;              // issued and not yet written
    bool stop = false;
    std::string error;
    std::thread thread;

    void run() {
        std::unique_lock<std::mutex> lock(mu);
        while (true) {
            cv.wait(lock, [&] { return stop || !ready.empty(); });
            if (ready.empty() && stop) return;
            SnapJob job = ready.front();
            ready.pop_front();
            lock.unlock();
            std::string err;
            FILE* f = std::fopen(job.path.c_str(), "wb");
            if (!f) {
                err = "sfgpu_save_raw: cannot open \"" + job.path + "\" for writing";
            } else {
                const size_t count = bytes / sizeof(float);
                if (std::fwrite(staging[job.buf], sizeof(float), count, f) != count)
                    err = "sfgpu_save_raw: short write to \"" + job.path + "\"";
                if (std::fclose(f) != 0 && err.empty()) err = "sfgpu_save_raw: closing \"" + job.path + "\" failed";
            }
            lock.lock();
            if (!err.empty() && error.empty()) error = err;
            busy[job.buf] = false;
            queued--;
            cv.notify_all();
        }
    }
};

namespace {

struct CallbackArg {
    SnapshotWriter* w;
    SnapJob job;
};

// Runs on a CUDA callback thread once the copy has landed: only hands the
// buffer over (no CUDA calls allowed here).
void CUDART_CB on_copied(void* p) {
    CallbackArg* a = (CallbackArg*)p;
    {
        std::lock_guard<std::mutex> lock(a->w->mu);
        a->w->ready.push_back(a->job);
    }
    a->w->cv.notify_all();
    delete a;
}

int writer_of(sfgpu_sim* s, SnapshotWriter** out) {
    if (!s->snap) {
        SnapshotWriter* w = new SnapshotWriter();
        w->bytes = sizeof(float) * (size_t)s->n * s->dof;
        for (int b = 0; b < SNAP_BUFFERS; b++) {
            if (cudaMallocHost(&w->staging[b], w->bytes ? w->bytes : 4) != cudaSuccess) {
                sf_set_error("snapshot: cannot allocate %zu bytes of page-locked staging memory", w->bytes);
                for (int k = 0; k < b; k++) cudaFreeHost(w->staging[k]);
                delete w;
                return SFGPU_FAILURE;
            }
        }
        w->thread = std::thread([w] { w->run(); });
        s->snap = w;
    }
    *out = s->snap;
    return SFGPU_OK;
}

}  // namespace

void sf_snapshot_free(sfgpu_sim* s) {
    SnapshotWriter* w = s->snap;
    if (!w) return;
    if (s->stream) cudaStreamSynchronize(s->stream);  // every callback has run
    {
        std::lock_guard<std::mutex> lock(w->mu);
        w->stop = true;
    }
    w->cv.notify_all();
    if (w->thread.joinable()) w->thread.join();
    for (int b = 0; b < SNAP_BUFFERS; b++) cudaFreeHost(w->staging[b]);
    delete w;
    s->snap = nullptr;
}

extern "C" int sfgpu_save_raw(sfgpu_sim* s, const char* filename) {
    sf_clear_error();
    if (!s || !filename) {
        sf_set_error("sfgpu_save_raw: %s is NULL", s ? "filename" : "simulation");
        return SFGPU_FAILURE;
    }
    SnapshotWriter* w = nullptr;
    if (writer_of(s, &w) != SFGPU_OK) return SFGPU_FAILURE;
    int buf = -1;
    {
        std::unique_lock<std::mutex> lock(w->mu);
        w->cv.wait(lock, [&] { return !w->busy[0] || !w->busy[1]; });
        buf = w->busy[0] ? 1 : 0;
        w->busy[buf] = true;
        w->queued++;
    }
    auto release = [&] {
        std::lock_guard<std::mutex> lock(w->mu);
        w->busy[buf] = false;
        w->queued--;
        w->cv.notify_all();
    };
    if (cudaMemcpyAsync(w->staging[buf], s->slab, w->bytes, cudaMemcpyDeviceToHost, s->stream) != cudaSuccess) {
        release();
        sf_set_error("sfgpu_save_raw: device-to-host copy failed: %s", cudaGetErrorString(cudaGetLastError()));
        return SFGPU_FAILURE;
    }
    CallbackArg* a = new CallbackArg{w, SnapJob{buf, filename}};
    if (cudaLaunchHostFunc(s->stream, on_copied, a) != cudaSuccess) {
        delete a;
        cudaStreamSynchronize(s->stream);
        release();
        sf_set_error("sfgpu_save_raw: cannot queue the writer: %s", cudaGetErrorString(cudaGetLastError()));
        return SFGPU_FAILURE;
    }
    return SFGPU_OK;
}

extern "C" int sfgpu_snapshot_wait(sfgpu_sim* s) {
    sf_clear_error();
    if (!s) {
        sf_set_error("sfgpu_snapshot_wait: simulation is NULL");
        return SFGPU_FAILURE;
    }
    SnapshotWriter* w = s->snap;
    if (!w) return SFGPU_OK;
    std::unique_lock<std::mutex> lock(w->mu);
    w->cv.wait(lock, [&] { return w->queued == 0; });
    if (!w->error.empty()) {
        sf_set_error("%s", w->error.c_str());
        w->error.clear();
        return SFGPU_FAILURE;
    }
    return SFGPU_OK;
}

extern "C" int sfgpu_read_raw(sfgpu_sim* s, const char* filename) {
    sf_clear_error();
    if (!s || !filename) {
        sf_set_error("sfgpu_read_raw: %s is NULL", s ? "filename" : "simulation");
        return SFGPU_FAILURE;
    }
    SnapshotWriter* w = nullptr;
    if (writer_of(s, &w) != SFGPU_OK) return SFGPU_FAILURE;
    // pending snapshots may still be reading the staging buffers
    if (sfgpu_snapshot_wait(s) != SFGPU_OK) return SFGPU_FAILURE;
    FILE* f = std::fopen(filename, "rb");
    if (!f) {
        sf_set_error("sfgpu_read_raw: cannot open \"%s\"", filename);
        return SFGPU_FAILURE;
    }
    const size_t count = w->bytes / sizeof(float);
    const size_t got = std::fread(w->staging[0], sizeof(float), count, f);
    std::fclose(f);
    if (got != count) {
        sf_set_error("sfgpu_read_raw: \"%s\" holds %zu of the %zu values of the slab", filename, got, count);
        return SFGPU_FAILURE;
    }
    return sfgpu_upload(s, w->staging[0]);
}
