// Asynchronous wavefield snapshot export (FdmSolver::exportSnapshot,
// solver/fdm.h:312-347, without its blocking copies).
//
// The reference copies each snapshot field to pageable host memory and writes
// its file before the next time step is launched. Here a snapshot is a
// device-to-device copy into a ring of staging buffers on the solver's
// stream (a few microseconds at HBM speed), then a device-to-host copy into
// a pinned buffer of the same ring slot on a side stream, and a writer
// thread that waits for that copy and writes the file while the time loop
// goes on. A ring slot is reused only after its file is written; when every
// slot is in flight, push() waits for the oldest one. drain() waits for every
// pending file, so a pass that returns has written all its snapshots.
#pragma once

#include <cuda_runtime.h>

#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace gb {

class SnapWriter {
public:
    static constexpr int kSlots = 8;

    SnapWriter() = default;
    SnapWriter(const SnapWriter &) = delete;
    SnapWriter &operator=(const SnapWriter &) = delete;
    ~SnapWriter() { close(); }

    // Buffers for fields of n floats on the current device (reallocated when n
    // changes). Returns a CUDA error code.
    cudaError_t open(size_t n);
    // Enqueues the export of d_src[0..n) (on stream st, at its current point)
    // to `file` in the model-file format.
    cudaError_t push(cudaStream_t st, const float *d_src, const std::string &file);
    // Waits until every pushed snapshot is written. Returns 0, or the first
    // error (a failed copy or file) with its message in *msg.
    int drain(std::string *msg);
    void close();

private:
    struct Job {
        int slot;
        std::string file;
    };
    void run();

    size_t n_ = 0;
    int device_ = 0;
    cudaStream_t st_io_ = nullptr;
    float *dstage_[kSlots] = {};
    float *hpin_[kSlots] = {};
    cudaEvent_t staged_[kSlots] = {}, copied_[kSlots] = {};
    bool busy_[kSlots] = {};
    int next_ = 0, pending_ = 0;
    std::deque<Job> jobs_;
    std::mutex m_;
    std::condition_variable cv_;
    std::thread worker_;
    bool stop_ = false;
    int err_ = 0;
    std::string errmsg_;
};

}  // namespace gb
