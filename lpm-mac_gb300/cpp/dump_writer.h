// Asynchronous writer of the LAMMPS dump that Assembly::writeDump appends
// after every load step (assembly.h:309-335 of the reference).  The caller
// hands over a copy of the particle columns and goes on; one worker thread
// formats the records and appends them in call order, with the reference's
// header and number format, so the file is the same byte for byte.  At most
// kMaxPending records wait at a time (a caller that would exceed it blocks);
// flush() returns once every record handed over is written, and the writer
// flushes when the program ends.  LPM_DUMP_SYNC=1 writes on the calling
// thread instead.
#pragma once

#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

// One writeDump call: the header fields and, per particle, id, type and the
// 15 columns x y z dx dy dz s11 s22 s33 s23 s13 s12 damage damage_visual
// state_var[0].
struct DumpRecord {
  std::string file;
  int step = 0, nparticle = 0;
  double box[6] = {0, 0, 0, 0, 0, 0};
  std::vector<int> id, type;
  std::vector<double> cols;
};

class DumpWriter {
 public:
  static constexpr int kCols = 15;
  static constexpr size_t kMaxPending = 4;

  static DumpWriter& instance() {
    static DumpWriter w;
    return w;
  }

  void submit(DumpRecord&& r) {
    if (sync_) {
      write(r);
      return;
    }
    std::unique_lock<std::mutex> lk(mu_);
    space_.wait(lk, [&] { return queue_.size() < kMaxPending; });
    queue_.push_back(std::move(r));
    ready_.notify_one();
  }

  // Blocks until every record handed over is on disk.
  void flush() {
    std::unique_lock<std::mutex> lk(mu_);
    idle_.wait(lk, [&] { return queue_.empty() && !busy_; });
  }

  ~DumpWriter() {
    flush();
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    ready_.notify_all();
    if (worker_.joinable()) worker_.join();
  }

  static void write(const DumpRecord& r) {
    FILE* f = fopen(r.file.c_str(), "a+");
    if (!f) return;
    fprintf(f, "ITEM: TIMESTEP\n%d\nITEM: NUMBER OF ATOMS\n%d\nITEM: BOX BOUNDS pp pp pp\n", r.step, r.nparticle);
    fprintf(f, "%8.8f %8.8f\n%8.8f %8.8f\n%8.8f %8.8f\n", r.box[0], r.box[1], r.box[2], r.box[3], r.box[4], r.box[5]);
    fprintf(f, "ITEM: ATOMS id type x y z dx dy dz s11 s22 s33 s23 s13 s12 damage damage_visual state_var[0] \n");
    for (size_t i = 0; i < r.id.size(); ++i) {
      const double* c = &r.cols[i * kCols];
      fprintf(f, "%d %d %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e %.4e\n", r.id[i],
              r.type[i], c[0], c[1], c[2], c[3], c[4], c[5], c[6], c[7], c[8], c[9], c[10], c[11], c[12], c[13],
              c[14]);
    }
    fclose(f);
  }

 private:
  DumpWriter() {
    const char* e = getenv("LPM_DUMP_SYNC");
    sync_ = e && strcmp(e, "0") != 0;
    if (!sync_) worker_ = std::thread([this] { run(); });
  }

  void run() {
    for (;;) {
      DumpRecord r;
      {
        std::unique_lock<std::mutex> lk(mu_);
        ready_.wait(lk, [&] { return stop_ || !queue_.empty(); });
        if (queue_.empty()) return;  // stopping, nothing left
        r = std::move(queue_.front());
        queue_.pop_front();
        busy_ = true;
        space_.notify_all();
      }
      write(r);
      {
        std::lock_guard<std::mutex> lk(mu_);
        busy_ = false;
      }
      idle_.notify_all();
    }
  }

  std::mutex mu_;
  std::condition_variable ready_, space_, idle_;
  std::deque<DumpRecord> queue_;
  std::thread worker_;
  bool busy_ = false, stop_ = false, sync_ = false;
};

// Waits until every dump handed to the writer is on disk (before reading a
// dump file back in the same program).
inline void flushDumps() { DumpWriter::instance().flush(); }
