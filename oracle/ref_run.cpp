// ref_run.cpp - runs the REFERENCE's own program (src/main.cpp compiled in
// place, its main renamed) on a parfile, with the HDF5 stand-in of
// shim/H5Cpp.h keeping in memory what it reads and writes: a caller puts the
// ejecta initial data there (what the reference's Python front end would write
// to id_a.h5), runs the program, and reads back what it wrote - the blastwave
// dynamics (saveEjectaBWsDynamics), the comoving spectra
// (computeSaveEjectaSpectrum) and the light curves (computeSaveEjectaLightCurve).
//
// Test infrastructure only: built by oracle/Makefile (target ref) into
// oracle/_ref/libpbaref_run.so when the reference sources are present, used by
// tests/golden/make_reference_run.py to record the reference driver's inputs
// and outputs. Nothing in the product links it.
#define main pbag_reference_main
#include "main.cpp"
#undef main

#include <csignal>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include <fcntl.h>
#include <sys/wait.h>
#include <unistd.h>

extern "C" {

// the store of the HDF5 stand-in
void ref_h5_put(const char* file, const char* name, const double* data, const unsigned long long* dims, int ndims) {
  std::vector<unsigned long long> d(dims, dims + ndims);
  size_t n = ndims ? 1 : 0;
  for (unsigned long long x : d) n *= (size_t)x;
  pbag_h5::put(file, name, std::vector<double>(data, data + n), d);
}
void ref_h5_put_attr(const char* file, const char* name, double v) { pbag_h5::put_attr(file, name, v); }
void ref_h5_clear() {
  pbag_h5::datasets().clear();
  pbag_h5::attributes().clear();
}
int ref_h5_count() { return (int)pbag_h5::datasets().size(); }
// key of dataset i (NUL-terminated into buf of len bytes); its element count
long ref_h5_key(int i, char* buf, int len) {
  auto it = pbag_h5::datasets().begin();
  std::advance(it, i);
  std::strncpy(buf, it->first.c_str(), (size_t)len - 1);
  buf[len - 1] = 0;
  return (long)it->second.data.size();
}
int ref_h5_get(const char* key, double* out) {
  const pbag_h5::Entry* e = pbag_h5::find(key);
  if (!e) return -1;
  std::memcpy(out, e->data.data(), e->data.size() * sizeof(double));
  return 0;
}
double ref_h5_get_attr(const char* key, int* found) {
  auto it = pbag_h5::attributes().find(key);
  *found = it != pbag_h5::attributes().end();
  return *found ? it->second : 0.;
}

}  // extern "C"

namespace {

const char* g_dump_path = nullptr;

// the store as a flat file: per dataset its key, rank, dims and values; then
// per attribute its key and value. Plain write(2) and no allocation, so that
// it also runs from the handler of the abort below (the heap is then not
// usable).
void dump_store(const char* path) {
  const int fd = ::open(path, O_WRONLY | O_CREAT | O_TRUNC, 0644);
  if (fd < 0) return;
  auto put = [&](const void* p, size_t n) {
    const char* c = static_cast<const char*>(p);
    while (n > 0) {
      const ssize_t w = ::write(fd, c, n);
      if (w <= 0) return;
      c += w;
      n -= (size_t)w;
    }
  };
  auto put_str = [&](const std::string& k) {
    const uint32_t n = (uint32_t)k.size();
    put(&n, sizeof n);
    put(k.data(), n);
  };
  const uint64_t nd = pbag_h5::datasets().size(), na = pbag_h5::attributes().size();
  put(&nd, sizeof nd);
  for (const auto& kv : pbag_h5::datasets()) {
    put_str(kv.first);
    const uint32_t rank = (uint32_t)kv.second.dims.size();
    put(&rank, sizeof rank);
    put(kv.second.dims.data(), sizeof(unsigned long long) * rank);
    const uint64_t n = kv.second.data.size();
    put(&n, sizeof n);
    put(kv.second.data.data(), sizeof(double) * n);
  }
  put(&na, sizeof na);
  for (const auto& kv : pbag_h5::attributes()) {
    put_str(kv.first);
    put(&kv.second, sizeof(double));
  }
  ::close(fd);
}

// the reference program's exit path frees one of its strings twice after
// its last output is written; the store is saved when that aborts it
void on_fatal(int sig) {
  if (g_dump_path) dump_store(g_dump_path);
  _exit(128 + sig);
}

}  // namespace

extern "C" {

// Runs the reference program (argv = {name, working_dir, parfile, loglevel})
// in a child process and saves the store it leaves to out_path (dump_store's
// format). Returns the child's exit status (0, or 128 + the signal that ended
// it after its outputs were written).
int ref_run(const char* working_dir, const char* parfile, const char* loglevel, const char* out_path) {
  std::fflush(nullptr);
  const pid_t pid = fork();
  if (pid < 0) return -1;
  if (pid == 0) {
    g_dump_path = out_path;
    std::signal(SIGSEGV, on_fatal);
    std::signal(SIGABRT, on_fatal);
    char a0[] = "pba.out";
    std::string w(working_dir), p(parfile), l(loglevel);
    char* argv[] = {a0, w.data(), p.data(), l.data(), nullptr};
    const int rc = pbag_reference_main(4, argv);
    dump_store(out_path);
    std::fflush(nullptr);
    _exit(rc);
  }
  int status = 0;
  if (waitpid(pid, &status, 0) < 0) return -1;
  return WIFEXITED(status) ? WEXITSTATUS(status) : 128 + WTERMSIG(status);
}

}  // extern "C"
