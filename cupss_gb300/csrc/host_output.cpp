// Output path of the drop-in API: the CSV field files of writeOut and the background
// writer that lets the time step continue while they are written.
//
// File format (src/field.cpp:350-402 of the reference): data/<name>.csv.<step>, a header
// "x, [y, [z, ]]<name>", then one line per grid point in index order k*sx*sy + j*sx + i:
// the integer coordinates and the value with writePrecision decimals, all separated by
// ", ".  A NaN value is an error (the reference prints "NaN found in field <name>" and
// exits with status 1).
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/cupss_gb300.h"
#include "host_common.h"

namespace cupssgb_host {

std::string write_field_csv(const std::string& path, const std::string& name, const float* v, int sx, int sy,
                            int sz, int dim, int precision) {
  FILE* fp = std::fopen(path.c_str(), "w+");
  if (!fp) return "Error creating output file " + path;
  std::vector<char> buf(1 << 20);
  std::setvbuf(fp, buf.data(), _IOFBF, buf.size());
  const std::string head = dim == 1 ? "x, " : (dim == 2 ? "x, y, " : "x, y, z, ");
  std::fprintf(fp, "%s%s\n", head.c_str(), name.c_str());
  std::string fmt = dim == 1 ? "%i, " : (dim == 2 ? "%i, %i, " : "%i, %i, %i, ");
  fmt += "%." + std::to_string(precision) + "f\n";
  std::string err;
  size_t idx = 0;
  for (int k = 0; k < sz && err.empty(); ++k)
    for (int j = 0; j < sy && err.empty(); ++j)
      for (int i = 0; i < sx; ++i, ++idx) {
        const float x = v[idx];
        if (std::isnan(x)) {
          err = "NaN found in field " + name;
          break;
        }
        int w = 0;
        if (dim == 1) w = std::fprintf(fp, fmt.c_str(), i, x);
        else if (dim == 2) w = std::fprintf(fp, fmt.c_str(), i, j, x);
        else w = std::fprintf(fp, fmt.c_str(), i, j, k, x);
        if (w < 0) {
          err = "Error writing data to output file " + path;
          break;
        }
      }
  if (std::fclose(fp) != 0 && err.empty()) err = "Error writing data to output file " + path;
  return err;
}

// One queued file: the host copy of the field arrives in `buf` when `done` completes.
struct OutputJob {
  std::string path, name;
  int sx, sy, sz, dim, precision;
  float* buf;
  cudaEvent_t done;
};

struct OutputWriter::Impl {
  int device = 0;
  size_t npoints = 0;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<OutputJob> queue;
  std::vector<float*> free_bufs;
  std::vector<float*> all_bufs;
  std::vector<cudaEvent_t> free_events;
  int busy = 0;   // jobs taken by the worker and not yet finished
  bool stop = false;
  std::string error;   // first failure of a queued file
  std::thread worker;

  void run() {
    cudaSetDevice(device);
    for (;;) {
      OutputJob job;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return stop || !queue.empty(); });
        if (queue.empty()) return;
        job = queue.front();
        queue.pop_front();
        ++busy;
      }
      std::string err;
      const cudaError_t e = cudaEventSynchronize(job.done);
      if (e != cudaSuccess) err = std::string("output copy failed: ") + cudaGetErrorString(e);
      else err = write_field_csv(job.path, job.name, job.buf, job.sx, job.sy, job.sz, job.dim, job.precision);
      {
        std::lock_guard<std::mutex> lk(mu);
        if (!err.empty() && error.empty()) error = err;
        free_bufs.push_back(job.buf);
        free_events.push_back(job.done);
        --busy;
      }
      cv.notify_all();
    }
  }
};

OutputWriter::OutputWriter(int device, size_t npoints) : impl_(new Impl) {
  impl_->device = device;
  impl_->npoints = npoints;
  impl_->worker = std::thread([this] { impl_->run(); });
}

OutputWriter::~OutputWriter() {
  {
    std::lock_guard<std::mutex> lk(impl_->mu);
    impl_->stop = true;
  }
  impl_->cv.notify_all();
  if (impl_->worker.joinable()) impl_->worker.join();
  for (float* b : impl_->all_bufs) cupssgb_host_free(b);
  for (cudaEvent_t e : impl_->free_events) cudaEventDestroy(e);
  delete impl_;
}

int OutputWriter::acquire(float** buf, void** done) {
  std::unique_lock<std::mutex> lk(impl_->mu);
  // at most kMaxPending files in flight: further writeOuts wait for the oldest
  impl_->cv.wait(lk, [&] {
    return !impl_->free_bufs.empty() || (int)impl_->all_bufs.size() < kMaxPending;
  });
  if (impl_->free_bufs.empty()) {
    void* p = nullptr;
    const int rc = cupssgb_host_alloc((long long)(impl_->npoints * sizeof(float)), &p);
    if (rc != 0) return rc;
    impl_->all_bufs.push_back((float*)p);
    impl_->free_bufs.push_back((float*)p);
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return CUPSSGB_ERR_CUDA;
    impl_->free_events.push_back(e);
  }
  *buf = impl_->free_bufs.back();
  impl_->free_bufs.pop_back();
  *done = (void*)impl_->free_events.back();
  impl_->free_events.pop_back();
  return 0;
}

void OutputWriter::submit(const std::string& path, const std::string& name, int sx, int sy, int sz, int dim,
                          int precision, float* buf, void* done) {
  {
    std::lock_guard<std::mutex> lk(impl_->mu);
    impl_->queue.push_back(OutputJob{path, name, sx, sy, sz, dim, precision, buf, (cudaEvent_t)done});
  }
  impl_->cv.notify_all();
}

void OutputWriter::release(float* buf, void* done) {
  {
    std::lock_guard<std::mutex> lk(impl_->mu);
    impl_->free_bufs.push_back(buf);
    impl_->free_events.push_back((cudaEvent_t)done);
  }
  impl_->cv.notify_all();
}

std::string OutputWriter::flush() {
  std::unique_lock<std::mutex> lk(impl_->mu);
  impl_->cv.wait(lk, [&] { return impl_->queue.empty() && impl_->busy == 0; });
  std::string e;
  e.swap(impl_->error);
  return e;
}

std::string OutputWriter::error() {
  std::lock_guard<std::mutex> lk(impl_->mu);
  std::string e;
  e.swap(impl_->error);
  return e;
}

}  // namespace cupssgb_host
