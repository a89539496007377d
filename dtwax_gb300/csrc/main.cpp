// dtwx_main -- command-line drop-in for DTWax's `main <fast5_folder> <kmer_model> <ref.fasta>`
// (src/main.cu:53-318).
//
//   dtwx_main <read_folder> <kmer_model> <ref.fasta> [options]
//
// Prints the reference's 6-column log on stdout (src/main.cu:289-297):
//   Read_ID  QUERY_LEN  REF_LEN  sDTW score: fwd-strand  sDTW score: rev-strand
//   <idx>\t<read_id>\t<QUERY_LEN>\t<REF_LEN>\t<fwd>\t<rev>
// so src/ReadUntil/calc_classification_threshold.py and plot_realtime.py keep
// parsing it.  Timing goes to stderr.  The best end position, strand and call
// go to an optional side file (--side), one line per read:
//   <idx>\t<read_id>\t<score>\t<end_pos>\t<strand: + or ->\t<call: target|non-target|skipped>
//
// Reads: FAST5 needs HDF5, which this library is not linked against, so the folder holds
// one read per file as a 1-D numpy array (*.npy: int16 ADC or float32/float64
// pA) or as whitespace-separated text samples (*.txt).  The read id is the file
// name without its extension.  Files are taken in name order.
//
// Options:
//   --fp32             FP32 cells (default FP16 half2 with running-min offset)
//   --mixed            FP16 differences with FP32 path cost
//   --ref-del          REF_DEL recurrence (left predecessor; FP16 or, with --fp32, FP32 cells)
//   --threshold T      score below T calls "target" (default 194)
//   --adapter N        samples skipped at the read start (default 1952, ADAPTER_LEN)
//   --query-len N      samples aligned per read (default 2048, QUERY_LEN; 0 = rest)
//   --allow-short      align reads shorter than adapter + query-len (default: skip them)
//   --max-ref-len N    cap k-mer positions per strand (REF_LEN compatibility)
//   --concat           score one sequence fwd||rev instead of the two strands
//   --side FILE        write end position, strand and call per read
//
// Read Until FIFO mode, a drop-in for the reference's Read Until binary
// `main <kmer_model> <ref.fasta> <pipe>` (src/ru_main.cu:67-326, fed by
// src/ReadUntil/simulate_minion.py or ont_readuntil.py):
//
//   dtwx_main --fifo <kmer_model> <ref.fasta> <pipe> [--fp32|--mixed] [--ref-del] [--threshold T]
//             [--reads N] [--query-len N] [--batches N]
//
// reads batches of N (default 10) reads x query-len (default 2,048) unsigned
// 8-bit samples from the named pipe (generate_load_squiggle.hpp:303-343,
// PIPE_SIZE = 10 x 2,048 at ru_main.cu:131-132) and prints, per read and with no
// header, the line the reference prints (ru_main.cu:304-310):
//   <idx>\t<idx>\t<QUERY_LEN>\t<REF_LEN>\t<fwd>\t<rev>
// flushing after every batch.  The reference's writers open the pipe, write
// part of a batch and close it again (ont_readuntil.py:49-50 writes 16,000
// bytes per open; simulate_minion.py reopens in its loop), and its reader
// reopens the pipe for every batch (generate_load_squiggle.hpp:94-106 inside
// the while (true) of ru_main.cu:172-179).  So here a writer closing the pipe
// ends nothing: the reader reopens it and keeps filling the current batch from
// the next writer.  Like the reference it runs until it is stopped: SIGINT or
// SIGTERM ends it cleanly between reads (exit status 0), and --batches N stops
// it after N whole batches.  Bytes of an unfinished batch are dropped.
#include <dirent.h>
#include <errno.h>
#include <fcntl.h>
#include <signal.h>
#include <unistd.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "dtwx.h"

namespace {

bool ends_with(const std::string &s, const std::string &suf) {
  return s.size() >= suf.size() && s.compare(s.size() - suf.size(), suf.size(), suf) == 0;
}

// Minimal .npy reader for 1-D little-endian int16/int32/float32/float64 arrays.
bool load_npy(const std::string &path, std::vector<float> &out, std::string &err) {
  std::ifstream f(path, std::ios::binary);
  if (!f) {
    err = "cannot open";
    return false;
  }
  char magic[6];
  f.read(magic, 6);
  if (!f || memcmp(magic, "\x93NUMPY", 6) != 0) {
    err = "not a .npy file";
    return false;
  }
  unsigned char ver[2];
  f.read(reinterpret_cast<char *>(ver), 2);
  uint32_t hlen = 0;
  if (ver[0] == 1) {
    unsigned char b[2];
    f.read(reinterpret_cast<char *>(b), 2);
    hlen = b[0] | (b[1] << 8);
  } else {
    unsigned char b[4];
    f.read(reinterpret_cast<char *>(b), 4);
    hlen = b[0] | (b[1] << 8) | (b[2] << 16) | ((uint32_t)b[3] << 24);
  }
  std::string header(hlen, '\0');
  f.read(&header[0], hlen);
  if (!f) {
    err = "truncated header";
    return false;
  }
  auto field = [&](const char *key) -> std::string {
    size_t p = header.find(key);
    if (p == std::string::npos) return "";
    p = header.find(':', p);
    if (p == std::string::npos) return "";
    ++p;
    while (p < header.size() && header[p] == ' ') ++p;
    size_t e = p;
    if (header[p] == '\'') {
      e = header.find('\'', p + 1);
      return header.substr(p + 1, e - p - 1);
    }
    if (header[p] == '(') {
      e = header.find(')', p);
      return header.substr(p + 1, e - p - 1);
    }
    while (e < header.size() && header[e] != ',' && header[e] != '}') ++e;
    return header.substr(p, e - p);
  };
  const std::string descr = field("'descr'");
  const std::string fortran = field("'fortran_order'");
  const std::string shape = field("'shape'");
  if (fortran.find("True") != std::string::npos) {
    err = "fortran order not supported";
    return false;
  }
  size_t n = 0;
  {
    std::string s = shape;
    s.erase(std::remove(s.begin(), s.end(), ' '), s.end());
    if (!s.empty() && s.back() == ',') s.pop_back();
    if (s.find(',') != std::string::npos) {
      err = "expected a 1-D array";
      return false;
    }
    n = s.empty() ? 1 : (size_t)std::stoull(s);
  }
  out.resize(n);
  auto read_as = [&](auto tag) {
    using T = decltype(tag);
    std::vector<T> tmp(n);
    f.read(reinterpret_cast<char *>(tmp.data()), sizeof(T) * n);
    for (size_t i = 0; i < n; ++i) out[i] = (float)tmp[i];
    return (bool)f;
  };
  bool ok = false;
  if (descr == "<i2")
    ok = read_as(int16_t());
  else if (descr == "<i4")
    ok = read_as(int32_t());
  else if (descr == "<f4")
    ok = read_as(float());
  else if (descr == "<f8")
    ok = read_as(double());
  else {
    err = "unsupported dtype " + descr;
    return false;
  }
  if (!ok) err = "truncated data";
  return ok;
}

bool load_txt(const std::string &path, std::vector<float> &out, std::string &err) {
  std::ifstream f(path);
  if (!f) {
    err = "cannot open";
    return false;
  }
  out.clear();
  double v;
  while (f >> v) out.push_back((float)v);
  if (!f.eof()) {
    err = "non-numeric sample";
    return false;
  }
  return true;
}

volatile sig_atomic_t g_fifo_stop = 0;
void fifo_on_signal(int) { g_fifo_stop = 1; }

// The Read Until FIFO loop (see the header comment).
int run_fifo(int argc, char **argv) {
  if (argc < 5) {
    std::cerr << "usage: dtwx_main --fifo <kmer_model> <ref.fasta> <pipe> [--fp32|--mixed] [--ref-del]\n"
                 "       [--threshold T] [--reads N] [--query-len N] [--batches N]\n";
    return 2;
  }
  long max_batches = 0;
  const std::string model = argv[2], fasta = argv[3], pipe_path = argv[4];
  dtwx_config cfg;
  dtwx_config_default(&cfg);
  int n_reads = 10, qlen = 2048;
  for (int i = 5; i < argc; ++i) {
    const std::string a = argv[i];
    auto next = [&](void) -> const char * {
      if (i + 1 >= argc) {
        std::cerr << "missing value for " << a << "\n";
        exit(2);
      }
      return argv[++i];
    };
    if (a == "--fp32")
      cfg.precision = DTWX_FP32;
    else if (a == "--mixed")
      cfg.precision = DTWX_MIXED;
    else if (a == "--ref-del")
      cfg.recurrence = DTWX_REF_DEL;
    else if (a == "--threshold")
      cfg.threshold = (float)atof(next());
    else if (a == "--reads")
      n_reads = atoi(next());
    else if (a == "--query-len")
      qlen = atoi(next());
    else if (a == "--batches")
      max_batches = atol(next());
    else {
      std::cerr << "unknown option " << a << "\n";
      return 2;
    }
  }
  if (n_reads <= 0 || qlen <= 0 || max_batches < 0) {
    std::cerr << "--reads and --query-len must be positive\n";
    return 2;
  }
  dtwx_handle *h = nullptr;
  if (dtwx_create(&cfg, model.c_str(), nullptr, fasta.c_str(), &h) != DTWX_OK) {
    std::cerr << "dtwx_create: " << dtwx_last_error(nullptr) << "\n";
    return 1;
  }
  const int64_t ref_len = dtwx_ref_len(h);
  // no SA_RESTART: a signal interrupts a blocked open() or read() (EINTR)
  struct sigaction sa;
  memset(&sa, 0, sizeof(sa));
  sa.sa_handler = fifo_on_signal;
  sigemptyset(&sa.sa_mask);
  sigaction(SIGINT, &sa, nullptr);
  sigaction(SIGTERM, &sa, nullptr);
  const size_t batch = (size_t)n_reads * (size_t)qlen;
  std::vector<char> buf(batch);
  std::vector<float> raw(batch);
  std::vector<int64_t> offsets((size_t)n_reads + 1);
  for (int r = 0; r <= n_reads; ++r) offsets[r] = (int64_t)r * qlen;
  std::vector<dtwx_result> res((size_t)n_reads);
  int rc = 0;
  int fd = -1;
  size_t have = 0;
  long batches = 0;
  while (!g_fifo_stop) {
    if (fd < 0) {
      // blocks until a writer opens the pipe
      fd = open(pipe_path.c_str(), O_RDONLY);
      if (fd < 0) {
        if (errno == EINTR) continue;
        std::cerr << "cannot open " << pipe_path << ": " << strerror(errno) << "\n";
        rc = 1;
        break;
      }
    }
    const ssize_t k = read(fd, buf.data() + have, batch - have);
    if (k < 0) {
      if (errno == EINTR) continue;
      std::cerr << "read " << pipe_path << ": " << strerror(errno) << "\n";
      rc = 1;
      break;
    }
    if (k == 0) {
      // the writer closed the pipe: wait for the next one, keep the batch
      close(fd);
      fd = -1;
      continue;
    }
    have += (size_t)k;
    if (have < batch) continue;
    have = 0;
    for (size_t i = 0; i < batch; ++i) raw[i] = (float)(unsigned char)buf[i];
    if (dtwx_classify_batch(h, raw.data(), offsets.data(), n_reads, res.data()) != DTWX_OK) {
      std::cerr << "dtwx_classify_batch: " << dtwx_last_error(h) << "\n";
      rc = 1;
      break;
    }
    for (int j = 0; j < n_reads; ++j)
      std::cout << j << "\t" << j << "\t" << qlen << "\t" << ref_len << "\t" << res[j].score_fwd << "\t"
                << res[j].score_rev << "\n";
    std::cout.flush();
    if (max_batches && ++batches >= max_batches) break;
  }
  if (fd >= 0) close(fd);
  dtwx_destroy(h);
  return rc;
}

int usage() {
  std::cerr << "usage: dtwx_main <read_folder> <kmer_model> <ref.fasta> [--fp32|--mixed] [--ref-del] [--threshold T]\n"
               "       [--adapter N] [--query-len N] [--allow-short] [--max-ref-len N] [--concat] [--side FILE]\n";
  return 2;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc >= 2 && std::string(argv[1]) == "--fifo") return run_fifo(argc, argv);
  if (argc < 4) return usage();
  const std::string folder = argv[1], model = argv[2], fasta = argv[3];
  dtwx_config cfg;
  dtwx_config_default(&cfg);
  cfg.adapter_skip = 1952;
  cfg.query_len = 2048;
  cfg.require_full = 1;
  std::string side;
  for (int i = 4; i < argc; ++i) {
    const std::string a = argv[i];
    auto next = [&](void) -> const char * {
      if (i + 1 >= argc) {
        std::cerr << "missing value for " << a << "\n";
        exit(2);
      }
      return argv[++i];
    };
    if (a == "--fp32")
      cfg.precision = DTWX_FP32;
    else if (a == "--mixed")
      cfg.precision = DTWX_MIXED;
    else if (a == "--ref-del")
      cfg.recurrence = DTWX_REF_DEL;
    else if (a == "--threshold")
      cfg.threshold = (float)atof(next());
    else if (a == "--adapter")
      cfg.adapter_skip = atoi(next());
    else if (a == "--query-len")
      cfg.query_len = atoi(next());
    else if (a == "--allow-short")
      cfg.require_full = 0;
    else if (a == "--max-ref-len")
      cfg.max_ref_len = atoll(next());
    else if (a == "--concat")
      cfg.strand_mode = DTWX_STRANDS_CONCAT;
    else if (a == "--side")
      side = next();
    else
      return usage();
  }

  std::vector<std::string> files;
  DIR *d = opendir(folder.c_str());
  if (!d) {
    std::cerr << "Error opening folder '" << folder << "'\n";
    return 1;
  }
  while (dirent *e = readdir(d)) {
    const std::string n = e->d_name;
    if (ends_with(n, ".npy") || ends_with(n, ".txt") || ends_with(n, ".fast5")) files.push_back(n);
  }
  closedir(d);
  std::sort(files.begin(), files.end());

  std::vector<float> raw;
  std::vector<int64_t> offsets{0};
  std::vector<std::string> ids;
  for (const std::string &n : files) {
    if (ends_with(n, ".fast5")) {
      std::cerr << "skipping " << n << ": FAST5 needs HDF5, which dtwx_main is not linked against\n";
      continue;
    }
    std::vector<float> s;
    std::string err;
    const std::string path = folder + "/" + n;
    const bool ok = ends_with(n, ".npy") ? load_npy(path, s, err) : load_txt(path, s, err);
    if (!ok) {
      std::cerr << "skipping " << n << ": " << err << "\n";
      continue;
    }
    raw.insert(raw.end(), s.begin(), s.end());
    offsets.push_back((int64_t)raw.size());
    ids.push_back(n.substr(0, n.rfind('.')));
  }

  dtwx_handle *h = nullptr;
  int rc = dtwx_create(&cfg, model.c_str(), nullptr, fasta.c_str(), &h);
  if (rc != DTWX_OK) {
    std::cerr << "dtwx_create failed (" << rc << "): " << dtwx_last_error(nullptr) << "\n";
    return 1;
  }
  const int n_reads = (int)ids.size();
  std::vector<dtwx_result> res(n_reads);
  const double t0 = dtwx_now_ms();
  rc = dtwx_classify_batch(h, raw.data(), offsets.data(), n_reads, res.data());
  const double ms = dtwx_now_ms() - t0;
  if (rc != DTWX_OK) {
    std::cerr << "dtwx_classify_batch failed (" << rc << "): " << dtwx_last_error(h) << "\n";
    dtwx_destroy(h);
    return 1;
  }
  // the reference's throughput figure, hpc_helpers.hpp:93-100
  const double qlen = cfg.query_len > 0 ? cfg.query_len : 0;
  std::cerr << "TIMING: " << ms << " ms " << (qlen / (ms * 1e3)) * n_reads / 10 << " Mbps (classify_batch)\n";

  const int64_t ref_len = dtwx_ref_len(h);
  std::cout << "Read_ID\tQUERY_LEN\tREF_LEN\tsDTW score: fwd-strand\tsDTW score: rev-strand\n";
  int printed = 0;
  std::ofstream sf;
  if (!side.empty()) sf.open(side);
  for (int j = 0; j < n_reads; ++j) {
    const dtwx_result &r = res[j];
    if (sf) {
      sf << j << "\t" << ids[j] << "\t" << r.score << "\t" << r.end_pos << "\t" << (r.strand ? '-' : '+') << "\t"
         << (r.call < 0 ? "skipped" : (r.call ? "target" : "non-target")) << "\n";
    }
    if (r.call < 0) continue;  // the reference drops reads shorter than the window
    std::cout << printed++ << "\t" << ids[j] << "\t" << r.n_samples << "\t" << ref_len << "\t" << r.score_fwd
              << "\t" << r.score_rev << "\n";
  }
  dtwx_destroy(h);
  return 0;
}
