#include "host_util.h"

#include <fstream>
#include <sstream>

namespace dtwx {

bool read_file(const std::string &path, std::string &out) {
  std::ifstream f(path, std::ios::binary);
  if (!f.good()) return false;
  std::ostringstream ss;
  ss << f.rdbuf();
  out = ss.str();
  return true;
}

bool parse_fasta(const std::string &text, std::string &seq, std::string &name, std::string &err) {
  std::string cur_name, content;
  size_t pos = 0;
  const size_t N = text.size();
  while (pos < N) {
    size_t e = text.find('\n', pos);
    if (e == std::string::npos) e = N;
    std::string line = text.substr(pos, e - pos);
    pos = e + 1;
    if (!line.empty() && line.back() == '\r') line.pop_back();
    if (line.empty() || line[0] == '>') {
      // the open record (if any) ends here and is dropped: only a record
      // still open at the end of the file is kept
      cur_name.clear();
      if (!line.empty()) cur_name = line.substr(1);
      content.clear();
    } else if (!cur_name.empty()) {
      if (line.find(' ') != std::string::npos) {
        cur_name.clear();
        content.clear();
      } else {
        content += line;
      }
    }
  }
  // load_reference.hpp:193-206 keeps only the record still open at the end
  // of the file, so the last record wins and a trailing empty line loses it.
  if (cur_name.empty()) {
    err = "invalid FASTA: no sequence record open at end of file";
    return false;
  }
  name = cur_name;
  seq = content;
  if (seq.size() < 6) {
    err = "FASTA record shorter than one 6-mer";
    return false;
  }
  return true;
}

static int code_of(char c) {
  switch (c) {
    case 'A': return 0;
    case 'C': return 1;
    case 'G': return 2;
    case 'T': return 3;
    default: return -1;
  }
}

bool parse_kmer_model(const std::string &text, std::vector<double> &table, std::string &err) {
  table.assign(4096, 0.0);
  std::vector<char> seen(4096, 0);
  std::istringstream in(text);
  std::string line;
  int lineno = 0;
  while (std::getline(in, line)) {
    ++lineno;
    if (!line.empty() && line.back() == '\r') line.pop_back();
    if (line.empty()) continue;
    std::istringstream ls(line);
    std::string kmer;
    double mean = 0, sd = 0;
    if (!(ls >> kmer >> mean)) {
      err = "k-mer model line " + std::to_string(lineno) + ": expected 'KMER mean stdev'";
      return false;
    }
    ls >> sd;
    if (kmer.size() != 6) {
      // header lines such as "kmer level_mean ..." are skipped
      bool alpha = true;
      for (char c : kmer) alpha &= code_of(c) >= 0;
      if (!alpha) continue;
      err = "k-mer model line " + std::to_string(lineno) + ": k-mer length is not 6";
      return false;
    }
    int code = 0;
    bool ok = true;
    for (char c : kmer) {
      int b = code_of(c);
      ok &= b >= 0;
      code = code * 4 + (b & 3);
    }
    if (!ok) {
      err = "k-mer model line " + std::to_string(lineno) + ": non-ACGT k-mer '" + kmer + "'";
      return false;
    }
    table[code] = mean;
    seen[code] = 1;
  }
  for (int i = 0; i < 4096; ++i)
    if (!seen[i]) {
      err = "k-mer model is missing " + std::to_string(4096 - i) + " or more 6-mers";
      return false;
    }
  return true;
}

}  // namespace dtwx
