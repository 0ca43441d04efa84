// Asynchronous wavefield snapshot export (see gb_snapshot.h).
#include "gb_snapshot.h"

#include "gb_config.h"
#include "gbfwi.h"

namespace gb {

cudaError_t SnapWriter::open(size_t n) {
    if (n_ == n && st_io_) return cudaSuccess;
    close();
    cudaError_t e = cudaGetDevice(&device_);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st_io_, cudaStreamNonBlocking);
    for (int s = 0; s < kSlots && e == cudaSuccess; s++) {
        e = cudaMalloc(&dstage_[s], n * 4);
        if (e == cudaSuccess) e = cudaMallocHost(&hpin_[s], n * 4);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&staged_[s], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&copied_[s], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        close();
        return e;
    }
    n_ = n;
    stop_ = false;
    err_ = 0;
    errmsg_.clear();
    next_ = 0;
    pending_ = 0;
    worker_ = std::thread(&SnapWriter::run, this);
    return cudaSuccess;
}

cudaError_t SnapWriter::push(cudaStream_t st, const float *d_src, const std::string &file) {
    int s;
    {
        std::unique_lock<std::mutex> lk(m_);
        s = next_;
        cv_.wait(lk, [&] { return !busy_[s]; });  // its previous file is written
        busy_[s] = true;
        next_ = (next_ + 1) % kSlots;
        pending_++;
    }
    cudaError_t e = cudaMemcpyAsync(dstage_[s], d_src, n_ * 4, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaEventRecord(staged_[s], st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st_io_, staged_[s], 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hpin_[s], dstage_[s], n_ * 4, cudaMemcpyDeviceToHost, st_io_);
    if (e == cudaSuccess) e = cudaEventRecord(copied_[s], st_io_);
    std::lock_guard<std::mutex> lk(m_);
    if (e != cudaSuccess) {
        busy_[s] = false;
        pending_--;
        cv_.notify_all();
        return e;
    }
    jobs_.push_back({s, file});
    cv_.notify_all();
    return cudaSuccess;
}

void SnapWriter::run() {
    cudaSetDevice(device_);
    for (;;) {
        Job j;
        {
            std::unique_lock<std::mutex> lk(m_);
            cv_.wait(lk, [&] { return stop_ || !jobs_.empty(); });
            if (jobs_.empty()) return;  // stop requested and nothing left
            j = jobs_.front();
            jobs_.pop_front();
        }
        int rc = 0;
        std::string msg;
        const cudaError_t e = cudaEventSynchronize(copied_[j.slot]);
        if (e != cudaSuccess) {
            rc = GB_ERR_CUDA;
            msg = std::string("snapshot copy: ") + cudaGetErrorString(e);
        } else if (write_bin(j.file, hpin_[j.slot], n_)) {
            rc = GB_ERR_IO;
            msg = "cannot write " + j.file;
        }
        std::lock_guard<std::mutex> lk(m_);
        if (rc && !err_) {
            err_ = rc;
            errmsg_ = msg;
        }
        busy_[j.slot] = false;
        pending_--;
        cv_.notify_all();
    }
}

int SnapWriter::drain(std::string *msg) {
    std::unique_lock<std::mutex> lk(m_);
    cv_.wait(lk, [&] { return pending_ == 0; });
    const int rc = err_;
    if (rc && msg) *msg = errmsg_;
    err_ = 0;
    errmsg_.clear();
    return rc;
}

void SnapWriter::close() {
    if (worker_.joinable()) {
        {
            std::lock_guard<std::mutex> lk(m_);
            stop_ = true;
        }
        cv_.notify_all();
        worker_.join();
    }
    if (st_io_) cudaStreamSynchronize(st_io_);
    for (int s = 0; s < kSlots; s++) {
        cudaFree(dstage_[s]);
        cudaFreeHost(hpin_[s]);
        if (staged_[s]) cudaEventDestroy(staged_[s]);
        if (copied_[s]) cudaEventDestroy(copied_[s]);
        dstage_[s] = hpin_[s] = nullptr;
        staged_[s] = copied_[s] = nullptr;
        busy_[s] = false;
    }
    if (st_io_) cudaStreamDestroy(st_io_);
    st_io_ = nullptr;
    n_ = 0;
    jobs_.clear();
    pending_ = 0;
}

}  // namespace gb
