// trajectory.cu -- trajectory files in the reference's binary format
// (src/demo/nbody_io.hpp:4-22, read by scripts/nbody_io/bin_reader.py:4-18):
//   uint64 n_times, uint64 n_var, float64 softening,
//   then n_times records of (float64 t, n_var float64 state values),
// native little-endian.  The reference writes the file at the end from the
// states RawOutput kept in memory; here records are appended as the
// integrator delivers accepted states, by a background thread, and the
// header's n_times is patched on close.
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "gbode.h"

struct gb_trajectory_s {
  FILE* f = nullptr;
  uint64_t n_var = 0;
  uint64_t n_times = 0;
  double softening = 0.0;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<std::vector<double>> queue;  // each: t followed by n_var values
  std::vector<std::vector<double>> spare;
  bool stop = false;
  int io_error = 0;
  std::thread worker;
};

namespace {

void writer_loop(gb_trajectory_s* w) {
  for (;;) {
    std::vector<double> rec;
    {
      std::unique_lock<std::mutex> lock(w->mu);
      w->cv.wait(lock, [w] { return w->stop || !w->queue.empty(); });
      if (w->queue.empty()) return;  // stop requested and drained
      rec = std::move(w->queue.front());
      w->queue.pop_front();
    }
    if (fwrite(rec.data(), sizeof(double), rec.size(), w->f) != rec.size()) w->io_error = 1;
    std::lock_guard<std::mutex> lock(w->mu);
    w->spare.push_back(std::move(rec));
    w->cv.notify_all();
  }
}

}  // namespace

extern "C" int gb_trajectory_open(const char* path, int64_t n_var, double softening,
                                  gb_trajectory* out) {
  if (!path || !out || n_var < 1) return GB_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  FILE* f = fopen(path, "wb");
  if (!f) return GB_ERR_INVALID_ARGUMENT;
  auto* w = new gb_trajectory_s();
  w->f = f;
  w->n_var = (uint64_t)n_var;
  w->softening = softening;
  uint64_t zero = 0;
  double soft = softening;
  if (fwrite(&zero, 8, 1, f) != 1 || fwrite(&w->n_var, 8, 1, f) != 1 ||
      fwrite(&soft, 8, 1, f) != 1) {
    fclose(f);
    delete w;
    return GB_ERR_INVALID_ARGUMENT;
  }
  w->worker = std::thread(writer_loop, w);
  *out = w;
  return GB_OK;
}

// Queues one record; at most 64 records wait before the caller blocks.
extern "C" int gb_trajectory_append(gb_trajectory w, double t, const double* x_host) {
  if (!w || !x_host) return GB_ERR_INVALID_ARGUMENT;
  std::vector<double> rec;
  {
    std::unique_lock<std::mutex> lock(w->mu);
    w->cv.wait(lock, [w] { return w->queue.size() < 64; });
    if (!w->spare.empty()) {
      rec = std::move(w->spare.back());
      w->spare.pop_back();
    }
  }
  rec.resize(w->n_var + 1);
  rec[0] = t;
  std::memcpy(rec.data() + 1, x_host, w->n_var * sizeof(double));
  {
    std::lock_guard<std::mutex> lock(w->mu);
    w->queue.push_back(std::move(rec));
    w->n_times += 1;
  }
  w->cv.notify_all();
  return GB_OK;
}

// gb_save_fn adaptor: pass the writer as `user` to the integrator.
extern "C" void gb_trajectory_save(void* user, double t, const double* x_host, int64_t n_var) {
  auto* w = static_cast<gb_trajectory>(user);
  if (w && (uint64_t)n_var == w->n_var) gb_trajectory_append(w, t, x_host);
}

extern "C" int gb_trajectory_close(gb_trajectory w, int64_t* n_times) {
  if (!w) return GB_ERR_INVALID_ARGUMENT;
  {
    std::lock_guard<std::mutex> lock(w->mu);
    w->stop = true;
  }
  w->cv.notify_all();
  w->worker.join();
  int rc = w->io_error ? GB_ERR_INVALID_ARGUMENT : GB_OK;
  if (fseek(w->f, 0, SEEK_SET) != 0 || fwrite(&w->n_times, 8, 1, w->f) != 1)
    rc = GB_ERR_INVALID_ARGUMENT;
  if (fclose(w->f) != 0) rc = GB_ERR_INVALID_ARGUMENT;
  if (n_times) *n_times = (int64_t)w->n_times;
  delete w;
  return rc;
}
