// sep_io.cpp -- the filter's output files and the merge of several filter runs
// into one state set.
//
// Writers, byte for byte what the reference's stdio calls write:
//   psi.dat, psi-filt-<tid>-<jns>.dat: raw FP64 state blocks, no header
//     (filter/main.c:129-131, filter/filter.c:44-47);
//   eval.dat: "%ld %.16g %g\n" = index, E, sigma (filter/main.c:138-142);
//   eval-filt-<tid>-<jns>.dat: "%ld %.16g %.16g\n" = index, E, target
//     (filter/filter.c:37-41).
// State files reach 116 GB (2048 states of 192^3), so a team of threads
// writes them with positioned writes of 64 MiB pieces.
//
// Merge: the step between the filter and bse/ (combine_filter_outputs.py).
// All states of all runs are sorted by (E, sigma, run, index in the run);
// eval.par gets the new indices, psi.par the state blocks in that order and
// merge_manifest.txt the mapping.  The checks, their order and their messages
// follow the script (combine_filter_outputs.py:125-214, 238-284, 292-305);
// the state blocks are copied by a team of threads with positioned reads and
// writes instead of one sequential 1 MiB-chunk copy.
#include <fcntl.h>
#include <sys/stat.h>
#include <sys/time.h>
#include <sys/types.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cctype>
#include <cerrno>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sep_gb300.h"

namespace sep {
void set_error(const std::string& msg);
}

namespace {

constexpr size_t kPiece = size_t(64) << 20;  // bytes per positioned write of a state file
constexpr size_t kChunk = size_t(8) << 20;   // bytes per read/write of a merged state block

// The script's MergeError: inputs that cannot be merged (status SEP_ERR_ARG).
struct MergeError {
  std::string msg;
};
// An OSError the script does not catch (status SEP_ERR_IO).
struct IoError {
  std::string msg;
};

int io_threads() {
  const unsigned h = std::thread::hardware_concurrency();
  return (int)std::max(1u, std::min(16u, h));
}

template <typename F> void run_team(int n, F&& f) {
  std::vector<std::thread> team;
  for (int t = 1; t < n; ++t) team.emplace_back(f, t);
  f(0);
  for (auto& th : team) th.join();
}

// str() of Python's OSError for a failed call on a path
std::string os_error(int err, const std::string& path) {
  return "[Errno " + std::to_string(err) + "] " + std::strerror(err) + ": '" + path + "'";
}

bool pwrite_all(int fd, const char* p, size_t n, off_t off) {
  while (n > 0) {
    const ssize_t w = ::pwrite(fd, p, n, off);
    if (w < 0) {
      if (errno == EINTR) continue;
      return false;
    }
    p += w;
    n -= (size_t)w;
    off += w;
  }
  return true;
}

// reads n bytes; returns the number read (short only at end of file), -1 on error
ssize_t pread_all(int fd, char* p, size_t n, off_t off) {
  size_t got = 0;
  while (got < n) {
    const ssize_t r = ::pread(fd, p + got, n - got, off + (off_t)got);
    if (r < 0) {
      if (errno == EINTR) continue;
      return -1;
    }
    if (r == 0) break;
    got += (size_t)r;
  }
  return (ssize_t)got;
}

// Writes `bytes` from `data` to a new file at `path` (truncating), in pieces
// spread over a team of threads when the file is large.
void write_file(const std::string& path, const char* data, size_t bytes) {
  const int fd = ::open(path.c_str(), O_WRONLY | O_CREAT | O_TRUNC | O_CLOEXEC, 0666);
  if (fd < 0) throw IoError{os_error(errno, path)};
  const size_t pieces = (bytes + kPiece - 1) / kPiece;
  const int team = (int)std::min<size_t>((size_t)io_threads(), std::max<size_t>(1, pieces));
  std::atomic<size_t> next{0};
  std::atomic<int> err{0};
  run_team(team, [&](int) {
    for (size_t k = next++; k < pieces && err.load() == 0; k = next++) {
      const size_t off = k * kPiece, n = std::min(kPiece, bytes - off);
      if (!pwrite_all(fd, data + off, n, (off_t)off)) err = errno ? errno : EIO;
    }
  });
  const int e = err.load();
  if (::close(fd) != 0 && e == 0) throw IoError{os_error(errno, path)};
  if (e) throw IoError{os_error(e, path)};
}

// ---- text helpers: Python's str.split()/strip() whitespace (ASCII part) --
bool py_space(unsigned char c) {
  return c == ' ' || (c >= '\t' && c <= '\r') || (c >= 0x1c && c <= 0x1f);
}

std::vector<std::string> split_ws(const std::string& s) {
  std::vector<std::string> out;
  size_t i = 0;
  while (i < s.size()) {
    while (i < s.size() && py_space((unsigned char)s[i])) ++i;
    size_t j = i;
    while (j < s.size() && !py_space((unsigned char)s[j])) ++j;
    if (j > i) out.emplace_back(s, i, j - i);
    i = j;
  }
  return out;
}

// Lines as Python's text-mode iteration yields them (universal newlines:
// "\n", "\r\n" and "\r" end a line).
std::vector<std::string> text_lines(const std::string& s) {
  std::vector<std::string> out;
  size_t start = 0;
  for (size_t i = 0; i < s.size(); ++i) {
    if (s[i] == '\n' || s[i] == '\r') {
      out.emplace_back(s, start, i - start);
      if (s[i] == '\r' && i + 1 < s.size() && s[i + 1] == '\n') ++i;
      start = i + 1;
    }
  }
  if (start < s.size()) out.emplace_back(s, start, s.size() - start);
  return out;
}

bool is_digit(char c) { return c >= '0' && c <= '9'; }

// digit ("_"? digit)*, from s[i]; returns the end or npos
size_t digitpart(const std::string& s, size_t i) {
  if (i >= s.size() || !is_digit(s[i])) return std::string::npos;
  ++i;
  while (i < s.size()) {
    if (is_digit(s[i])) {
      ++i;
    } else if (s[i] == '_' && i + 1 < s.size() && is_digit(s[i + 1])) {
      i += 2;
    } else {
      break;
    }
  }
  return i;
}

std::string without_underscores(const std::string& s) {
  std::string t;
  for (char c : s)
    if (c != '_') t += c;
  return t;
}

// int(token) of Python (base 10): [+-] digitpart.  Values beyond long saturate.
bool py_int(const std::string& s, long* v) {
  size_t i = (!s.empty() && (s[0] == '+' || s[0] == '-')) ? 1 : 0;
  if (digitpart(s, i) != s.size()) return false;
  errno = 0;
  *v = std::strtol(without_underscores(s).c_str(), nullptr, 10);
  return true;
}

bool iequals(const std::string& a, const char* b) {
  const size_t n = std::strlen(b);
  if (a.size() != n) return false;
  for (size_t i = 0; i < n; ++i)
    if (std::tolower((unsigned char)a[i]) != b[i]) return false;
  return true;
}

// float(token) of Python: [+-] (pointfloat | exponentfloat | inf | infinity | nan)
bool py_float(const std::string& s, double* v) {
  size_t i = (!s.empty() && (s[0] == '+' || s[0] == '-')) ? 1 : 0;
  const std::string body = s.substr(i);
  if (iequals(body, "inf") || iequals(body, "infinity") || iequals(body, "nan")) {
    *v = std::strtod(s.c_str(), nullptr);
    return true;
  }
  bool mant = false;
  size_t j = digitpart(s, i);
  if (j != std::string::npos) {
    mant = true;
    i = j;
  }
  if (i < s.size() && s[i] == '.') {
    ++i;
    j = digitpart(s, i);
    if (j != std::string::npos) {
      mant = true;
      i = j;
    }
  }
  if (!mant) return false;
  if (i < s.size() && (s[i] == 'e' || s[i] == 'E')) {
    ++i;
    if (i < s.size() && (s[i] == '+' || s[i] == '-')) ++i;
    j = digitpart(s, i);
    if (j == std::string::npos) return false;
    i = j;
  }
  if (i != s.size()) return false;
  *v = std::strtod(without_underscores(s).c_str(), nullptr);
  return true;
}

// f"{x:.16g}" of Python (C's %.16g, with "nan" unsigned)
std::string g16(double x) {
  if (std::isnan(x)) return "nan";
  char b[64];
  std::snprintf(b, sizeof b, "%.16g", x);
  return b;
}

// ---- paths ---------------------------------------------------------------
std::vector<std::string> components(const std::string& p) {
  std::vector<std::string> out;
  size_t i = 0;
  while (i <= p.size()) {
    const size_t j = std::min(p.find('/', i), p.size());
    const std::string c = p.substr(i, j - i);
    if (!c.empty() && c != ".") out.push_back(c);
    i = j + 1;
  }
  return out;
}

std::string join_parts(const std::vector<std::string>& parts, bool absolute) {
  std::string s = absolute ? "/" : "";
  for (size_t k = 0; k < parts.size(); ++k) s += (k ? "/" : "") + parts[k];
  return s.empty() ? "." : s;
}

// root / name as pathlib joins them: an absolute name replaces the root,
// "." parts and repeated slashes drop out
std::string path_join(const std::string& root, const std::string& name) {
  if (!name.empty() && name[0] == '/') return join_parts(components(name), true);
  std::vector<std::string> parts = components(root);
  for (const std::string& c : components(name)) parts.push_back(c);
  return join_parts(parts, !root.empty() && root[0] == '/');
}

std::string parent_of(const std::string& p) {
  const size_t k = p.rfind('/');
  if (k == std::string::npos || k == 0) return "/";
  return p.substr(0, k);
}

// Path(p).resolve(): absolute, symbolic links resolved for the part that
// exists, the rest appended with ".." applied
std::string resolve(const std::string& p) {
  std::string abs = p;
  if (p.empty() || p[0] != '/') {
    char cwd[PATH_MAX];
    if (!::getcwd(cwd, sizeof cwd)) throw IoError{os_error(errno, ".")};
    abs = std::string(cwd) + "/" + p;
  }
  std::string cur = "/";
  bool exists = true;
  for (const std::string& c : components(abs)) {
    if (c == "..") {
      cur = parent_of(cur);
      continue;
    }
    const std::string next = cur == "/" ? "/" + c : cur + "/" + c;
    if (exists) {
      char buf[PATH_MAX];
      if (::realpath(next.c_str(), buf)) {
        cur = buf;
        continue;
      }
      exists = false;
    }
    cur = next;
  }
  return cur;
}

bool is_file(const std::string& p) {
  struct stat st;
  return ::stat(p.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}

// the whole file, or errno
int read_all(const std::string& path, std::string& out) {
  const int fd = ::open(path.c_str(), O_RDONLY | O_CLOEXEC);
  if (fd < 0) return errno;
  out.clear();
  char buf[1 << 16];
  for (;;) {
    const ssize_t r = ::read(fd, buf, sizeof buf);
    if (r < 0) {
      if (errno == EINTR) continue;
      const int e = errno;
      ::close(fd);
      return e;
    }
    if (r == 0) break;
    out.append(buf, (size_t)r);
  }
  ::close(fd);
  return 0;
}

// ---- the merge (combine_filter_outputs.py) -------------------------------
struct Row {
  long idx;
  double energy, sigma;
};

struct Dataset {
  std::string root, eval_path, psi_path, conf_path;  // conf_path empty when absent
  std::vector<Row> rows;
};

struct Record {
  double energy, sigma;
  long source, local;
};

// combine_filter_outputs.py:125-145
long read_ngrid(const std::string& path) {
  std::string text;
  if (const int e = read_all(path, text))
    throw MergeError{"failed to read grid source " + path + ": " + os_error(e, path)};
  const std::vector<std::string> tok = split_ws(text);
  if (tok.size() < 3) throw MergeError{"grid source " + path + " does not contain nx ny nz"};
  long n[3];
  for (int k = 0; k < 3; ++k)
    if (!py_int(tok[k], &n[k]))
      throw MergeError{"grid source " + path + " does not start with integer nx ny nz"};
  if (n[0] <= 0 || n[1] <= 0 || n[2] <= 0)
    throw MergeError{"grid source " + path + " contains a non-positive grid size"};
  return n[0] * n[1] * n[2];
}

// combine_filter_outputs.py:155-179
std::vector<Row> parse_eval(const std::string& path) {
  std::string text;
  if (const int e = read_all(path, text))
    throw MergeError{"failed to read " + path + ": " + os_error(e, path)};
  std::vector<Row> rows;
  const std::vector<std::string> lines = text_lines(text);
  for (size_t k = 0; k < lines.size(); ++k) {
    const std::vector<std::string> parts = split_ws(lines[k]);
    if (parts.empty()) continue;
    const std::string where = path + ":" + std::to_string(k + 1);
    if (parts.size() < 3) throw MergeError{where + " does not have 3 columns"};
    Row r;
    if (!py_int(parts[0], &r.idx) || !py_float(parts[1], &r.energy) ||
        !py_float(parts[2], &r.sigma))
      throw MergeError{where + " has a non-numeric field"};
    rows.push_back(r);
  }
  if (rows.empty()) throw MergeError{path + " is empty"};
  return rows;
}

// combine_filter_outputs.py:182-225
Dataset discover(const std::string& dir, const std::string& eval_name, const std::string& psi_name,
                 long ngrid) {
  Dataset d;
  d.root = resolve(dir);
  d.eval_path = path_join(d.root, eval_name);
  d.psi_path = path_join(d.root, psi_name);
  const std::string input_path = path_join(d.root, "input.par");
  const std::string conf_path = path_join(d.root, "conf.par");
  if (!is_file(d.eval_path)) throw MergeError{"missing " + d.eval_path};
  if (!is_file(d.psi_path)) throw MergeError{"missing " + d.psi_path};
  d.rows = parse_eval(d.eval_path);
  const long nstates = (long)d.rows.size();
  if (is_file(input_path)) {
    const long g = read_ngrid(input_path);
    if (g != ngrid)
      throw MergeError{input_path + " implies ngrid=" + std::to_string(g) + ", expected " +
                       std::to_string(ngrid)};
  }
  struct stat st;
  if (::stat(d.psi_path.c_str(), &st) != 0) throw IoError{os_error(errno, d.psi_path)};
  const long long expected = (long long)nstates * ngrid * (long long)sizeof(double);
  if ((long long)st.st_size != expected)
    throw MergeError{d.psi_path + " size is " + std::to_string((long long)st.st_size) +
                     " bytes, expected " + std::to_string(expected) + " for " +
                     std::to_string(nstates) + " states and ngrid=" + std::to_string(ngrid)};
  for (long k = 0; k < nstates; ++k)
    if (d.rows[k].idx != k)
      throw MergeError{d.eval_path + " indices are not sequential 0.." +
                       std::to_string(nstates - 1) +
                       "; the psi block mapping would be ambiguous"};
  if (is_file(conf_path)) d.conf_path = conf_path;
  return d;
}

// combine_filter_outputs.py:250-263 (the script compares SHA-256 digests;
// comparing the bytes decides the same)
void ensure_matching_conf(const std::vector<Dataset>& ds) {
  std::vector<const Dataset*> with;
  for (const Dataset& d : ds)
    if (!d.conf_path.empty()) with.push_back(&d);
  if (with.size() <= 1) return;
  std::string first, other;
  if (const int e = read_all(with[0]->conf_path, first))
    throw IoError{os_error(e, with[0]->conf_path)};
  for (size_t k = 1; k < with.size(); ++k) {
    if (const int e = read_all(with[k]->conf_path, other))
      throw IoError{os_error(e, with[k]->conf_path)};
    if (other != first)
      throw MergeError{"conf.par files differ between datasets; these filter outputs do not "
                       "describe the same nanostructure and cannot be merged for BSE"};
  }
}

// Python's tuple order on (energy, sigma, source, local): the first pair of
// fields that are not == decides by <.
bool record_less(const Record& a, const Record& b) {
  if (!(a.energy == b.energy)) return a.energy < b.energy;
  if (!(a.sigma == b.sigma)) return a.sigma < b.sigma;
  if (a.source != b.source) return a.source < b.source;
  return a.local < b.local;
}

// Stable bottom-up merge sort.  Every access stays in bounds whatever the
// comparison answers (a NaN energy makes the order partial).
void sort_records(std::vector<Record>& v) {
  std::vector<Record> tmp(v.size());
  for (size_t w = 1; w < v.size(); w *= 2) {
    for (size_t lo = 0; lo < v.size(); lo += 2 * w) {
      const size_t mid = std::min(lo + w, v.size()), hi = std::min(lo + 2 * w, v.size());
      size_t i = lo, j = mid, o = lo;
      while (i < mid && j < hi) tmp[o++] = record_less(v[j], v[i]) ? v[j++] : v[i++];
      while (i < mid) tmp[o++] = v[i++];
      while (j < hi) tmp[o++] = v[j++];
    }
    v.swap(tmp);
  }
}

void make_dirs(const std::string& path) {
  std::string cur = path[0] == '/' ? "" : ".";
  for (const std::string& c : components(path)) {
    cur += "/" + c;
    if (::mkdir(cur.c_str(), 0777) != 0 && errno != EEXIST) throw IoError{os_error(errno, cur)};
  }
  struct stat st;
  if (::stat(path.c_str(), &st) != 0) throw IoError{os_error(errno, path)};
  if (!S_ISDIR(st.st_mode)) throw IoError{os_error(EEXIST, path)};
}

// psi.par: block r of the output is block records[r].local of source records[r].source
void copy_blocks(const std::vector<Dataset>& ds, const std::vector<Record>& recs, long ngrid,
                 const std::string& out_path) {
  std::vector<int> fds;
  auto close_all = [&]() {
    for (int f : fds) ::close(f);
  };
  for (const Dataset& d : ds) {
    const int f = ::open(d.psi_path.c_str(), O_RDONLY | O_CLOEXEC);
    if (f < 0) {
      const int e = errno;
      close_all();
      throw IoError{os_error(e, d.psi_path)};
    }
    fds.push_back(f);
  }
  const int out = ::open(out_path.c_str(), O_WRONLY | O_CREAT | O_TRUNC | O_CLOEXEC, 0666);
  if (out < 0) {
    const int e = errno;
    close_all();
    throw IoError{os_error(e, out_path)};
  }
  const size_t block = (size_t)ngrid * sizeof(double);
  const size_t nrec = recs.size();
  const int team = (int)std::min<size_t>((size_t)io_threads(), std::max<size_t>(1, nrec));
  std::atomic<size_t> next{0};
  std::atomic<int> err{0};
  std::atomic<bool> short_read{false};
  run_team(team, [&](int) {
    std::vector<char> buf(std::min(kChunk, std::max<size_t>(block, 1)));
    for (size_t r = next++; r < nrec && err.load() == 0 && !short_read.load(); r = next++) {
      const int src = fds[recs[r].source];
      const off_t in0 = (off_t)((size_t)recs[r].local * block), out0 = (off_t)(r * block);
      for (size_t done = 0; done < block;) {
        const size_t n = std::min(buf.size(), block - done);
        const ssize_t got = pread_all(src, buf.data(), n, in0 + (off_t)done);
        if (got < 0) {
          err = errno ? errno : EIO;
          break;
        }
        if ((size_t)got < n) {
          short_read = true;
          break;
        }
        if (!pwrite_all(out, buf.data(), n, out0 + (off_t)done)) {
          err = errno ? errno : EIO;
          break;
        }
        done += n;
      }
    }
  });
  ::close(out);
  close_all();
  if (short_read.load())
    throw MergeError{"unexpected end of psi.dat while copying a state block"};
  if (err.load()) throw IoError{os_error(err.load(), out_path)};
}

// shutil.copy2: contents, permission bits and access/modification times
void copy_file_with_times(const std::string& src, const std::string& dst) {
  std::string data;
  if (const int e = read_all(src, data)) throw IoError{os_error(e, src)};
  write_file(dst, data.data(), data.size());
  struct stat st;
  if (::stat(src.c_str(), &st) == 0) {
    ::chmod(dst.c_str(), st.st_mode & 07777);
    struct timespec ts[2] = {st.st_atim, st.st_mtim};
    ::utimensat(AT_FDCWD, dst.c_str(), ts, 0);
  }
}

// combine_filter_outputs.py:266-312
void write_merge(const std::string& outdir, const std::vector<Dataset>& ds,
                 const std::vector<Record>& recs, long ngrid, bool copy_conf) {
  make_dirs(outdir);
  std::string ev;
  for (size_t r = 0; r < recs.size(); ++r)
    ev += std::to_string(r) + " " + g16(recs[r].energy) + " " + g16(recs[r].sigma) + "\n";
  write_file(path_join(outdir, "eval.par"), ev.data(), ev.size());
  copy_blocks(ds, recs, ngrid, path_join(outdir, "psi.par"));
  std::string man = "ngrid " + std::to_string(ngrid) + "\nnstates " +
                    std::to_string(recs.size()) + "\n";
  for (size_t k = 0; k < ds.size(); ++k)
    man += "source " + std::to_string(k) + " " + ds[k].root +
           " states=" + std::to_string(ds[k].rows.size()) + "\n";
  for (size_t r = 0; r < recs.size(); ++r)
    man += "merged_state " + std::to_string(r) + " source=" + std::to_string(recs[r].source) +
           " local_index=" + std::to_string(recs[r].local) + " energy=" + g16(recs[r].energy) +
           " sigma=" + g16(recs[r].sigma) + "\n";
  write_file(path_join(outdir, "merge_manifest.txt"), man.data(), man.size());
  if (copy_conf) {
    if (ds[0].conf_path.empty())
      throw MergeError{"--copy-conf was requested, but the first dataset has no conf.par"};
    copy_file_with_times(ds[0].conf_path, path_join(outdir, "conf.par"));
  }
}

int fail(int status, const std::string& msg) {
  sep::set_error(msg);
  return status;
}

std::string eval_lines(const char* fmt, const double* a, const double* b, long m) {
  std::string s;
  char line[160];
  for (long k = 0; k < m; ++k) {
    const int n = std::snprintf(line, sizeof line, fmt, k, a[k], b[k]);
    s.append(line, (size_t)std::max(0, std::min(n, (int)sizeof line - 1)));
  }
  return s;
}

template <typename F> int guarded(F&& f) {
  try {
    f();
    return SEP_OK;
  } catch (const MergeError& e) {
    return fail(SEP_ERR_ARG, e.msg);
  } catch (const IoError& e) {
    return fail(SEP_ERR_IO, e.msg);
  } catch (const std::exception& e) {
    return fail(SEP_ERR_IO, e.what());
  }
}

}  // namespace

extern "C" {

int sep_write_states(const char* path, const double* psi, long m, long ngrid) {
  if (!path || m < 0 || ngrid < 0 || (m * ngrid > 0 && !psi))
    return fail(SEP_ERR_ARG, "sep_write_states: bad arguments");
  return guarded([&] {
    write_file(path, reinterpret_cast<const char*>(psi), (size_t)m * (size_t)ngrid * sizeof(double));
  });
}

int sep_write_eval(const char* path, const double* eval, const double* sige, long m) {
  if (!path || m < 0 || (m > 0 && (!eval || !sige)))
    return fail(SEP_ERR_ARG, "sep_write_eval: bad arguments");
  return guarded([&] {
    const std::string s = eval_lines("%ld %.16g %g\n", eval, sige, m);
    write_file(path, s.data(), s.size());
  });
}

int sep_write_filter_eval(const char* path, const double* eval, const double* el, long ms) {
  if (!path || ms < 0 || (ms > 0 && (!eval || !el)))
    return fail(SEP_ERR_ARG, "sep_write_filter_eval: bad arguments");
  return guarded([&] {
    const std::string s = eval_lines("%ld %.16g %.16g\n", eval, el, ms);
    write_file(path, s.data(), s.size());
  });
}

int sep_read_grid_source(const char* path, long* ngrid) {
  if (!path || !ngrid) return fail(SEP_ERR_ARG, "sep_read_grid_source: bad arguments");
  return guarded([&] { *ngrid = read_ngrid(path); });
}

int sep_combine_outputs(int ndatasets, const char* const* dirs, const char* eval_name,
                        const char* psi_name, long ngrid, const char* output_dir, int copy_conf,
                        long* nstates, long* total) {
  if (ndatasets < 1 || !dirs) return fail(SEP_ERR_ARG, "sep_combine_outputs: no datasets");
  if (ngrid <= 0) return fail(SEP_ERR_ARG, "--ngrid must be positive");
  for (int k = 0; k < ndatasets; ++k)
    if (!dirs[k]) return fail(SEP_ERR_ARG, "sep_combine_outputs: null dataset path");
  const std::string en = eval_name ? eval_name : "eval.dat";
  const std::string pn = psi_name ? psi_name : "psi.dat";
  const std::string od = output_dir ? output_dir : "merged_filter";
  return guarded([&] {
    std::vector<Dataset> ds;
    for (int k = 0; k < ndatasets; ++k) ds.push_back(discover(dirs[k], en, pn, ngrid));
    ensure_matching_conf(ds);
    std::vector<Record> recs;
    for (size_t s = 0; s < ds.size(); ++s)
      for (size_t l = 0; l < ds[s].rows.size(); ++l)
        recs.push_back({ds[s].rows[l].energy, ds[s].rows[l].sigma, (long)s, (long)l});
    sort_records(recs);
    if (nstates)
      for (int k = 0; k < ndatasets; ++k) nstates[k] = (long)ds[k].rows.size();
    if (total) *total = (long)recs.size();
    write_merge(resolve(od), ds, recs, ngrid, copy_conf != 0);
  });
}

}  // extern "C"
