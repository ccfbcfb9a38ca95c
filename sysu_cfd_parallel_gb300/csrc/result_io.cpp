// Result files in the reference's formats (host side; the fields come off the device first).
//
//   tec/res%04d.dat   Output2Tecplot         NS/navierIO.cpp:161-283 (FEBRICK, BLOCK, ASCII)
//   tec/data          Output2TecplotBinary   NS/navierIO.cpp:132-159
//   tec/grid.dat      OutputGrid             NS/navierIO.cpp:58-128
//   tec/geo           OutputGridBinary       NS/navierIO.cpp:29-55
//   res.sav           WriteBackupFile / ReadBackupFile   NS/navierIO.cpp:370-404
//
// Every file is what one rank of the reference writes when it owns the whole mesh (rank 0 of
// one process: no interface vertices, partition header {0, 1}).  Numbers go through the C
// library's printf conversions, as the reference's sprintf and ostream do, so the text is the
// same byte for byte.  Compiled with -ffp-contract=off: the derived Mach column is rounded
// exactly as written.
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <functional>
#include <string>
#include <thread>
#include <vector>

#include "cycas_host.h"

namespace cycas {

namespace {

// OutArray2File (navierIO.cpp:2-17): each value rendered "%19.5f " on a fixed 20-character
// stride, "\n" after every fifth value, "\n" after the block.  A value wider than the stride
// (|x| >= 1e13) keeps its first 20 characters, because the next value or line break is written
// over the rest; only a last value that ends no line of five keeps its full width.  An empty
// block is the final "\n" alone.
void block(std::string& out, const double* a, long n, int stride) {
  char buf[512];
  for (long i = 0; i < n; i++) {
    int len = std::snprintf(buf, sizeof buf, "%19.5f ", a[i * (long)stride]);
    if (len < 0) len = 0;
    if (len > (int)sizeof buf - 1) len = (int)sizeof buf - 1;
    const bool fifth = (i % 5) == 4;
    if (len > 20 && (i != n - 1 || fifth)) len = 20;
    out.append(buf, (size_t)len);
    if (fifth) out.push_back('\n');
  }
  out.push_back('\n');
}

// Renders parts [0, nparts) with part(i, out_i) on up to the host's hardware threads and
// returns them in order; the text does not depend on the thread count.
std::vector<std::string> render_parts(int nparts, const std::function<void(int, std::string&)>& part) {
  std::vector<std::string> out((size_t)nparts);
  const int nt = std::max(1, std::min(nparts, (int)std::thread::hardware_concurrency()));
  std::atomic<int> next{0};
  auto work = [&]() {
    for (int i = next++; i < nparts; i = next++) part(i, out[(size_t)i]);
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; t++) pool.emplace_back(work);
  work();
  for (auto& th : pool) th.join();
  return out;
}

// cells [lo, hi) of chunk i of n cells cut into `chunks` pieces
void chunk_range(long n, int chunks, int i, long& lo, long& hi) {
  lo = n * i / chunks;
  hi = n * (i + 1) / chunks;
}

void append_i32(std::string& out, int32_t v) { out.append(reinterpret_cast<const char*>(&v), sizeof v); }

void append_f64(std::string& out, const double* a, long n) {
  out.append(reinterpret_cast<const char*>(a), sizeof(double) * (size_t)n);
}

}  // namespace

std::string tecplot_text(const double* vert, long nvrt, const int32_t* cell_vertices, const CellFieldsView& f) {
  const long n = f.ncel;
  const int nvar = f.turb == 1 ? 8 : 6;  // FlowField::nVar (BasicType.h:95-111)
  std::string out = "variables= \"x\", \"y\", \"z\", \"p\", \"u\", \"v\", \"w\", \"ro\", \"T\",\"Ma\",\"mu\" ";
  if (f.turb == 1) out += "\"te\", \"ed\"";
  out += "\n";
  char line[256];
  std::snprintf(line, sizeof line,
                "ZONE N=%ld, E=%ld, VARLOCATION=([1-3]=NODAL,[4-%d]=CELLCENTERED) DATAPACKING=BLOCK, "
                "ZONETYPE=FEBRICK\n",
                nvrt, n, 3 + nvar + 2);
  out += line;
  // blocks x y z, P U V W R T, Ma, mu, [TE ED], then the connectivity in chunks of cells; every
  // block is independent text, rendered in parallel and joined in order
  std::vector<double> ma((size_t)n), mu((size_t)n);
  for (long i = 0; i < n; i++) {  // Mach number (perfect gas) or velocity magnitude; VisLam + VisTur
    if (f.density == 1)
      ma[i] = std::sqrt((f.U[i] * f.U[i] + f.V[i] * f.V[i] + f.W[i] * f.W[i]) / (1.4 * (f.P[i] + f.pref) / f.R[i]));
    else
      ma[i] = std::sqrt((f.U[i] * f.U[i] + f.V[i] * f.V[i] + f.W[i] * f.W[i]));
    mu[i] = f.VisLam[i] + f.VisTur[i];
  }
  std::vector<const double*> cols = {f.P, f.U, f.V, f.W, f.R, f.T, ma.data(), mu.data()};
  if (f.turb == 1) {
    cols.push_back(f.TE);
    cols.push_back(f.ED);
  }
  const int nblocks = 3 + (int)cols.size(), conn_chunks = 16;
  std::vector<std::string> parts = render_parts(nblocks + conn_chunks, [&](int i, std::string& o) {
    if (i < 3) {
      o.reserve((size_t)nvrt * 21 + 2);
      block(o, vert + i, nvrt, 3);
    } else if (i < nblocks) {
      o.reserve((size_t)n * 21 + 2);
      block(o, cols[(size_t)(i - 3)], n, 1);
    } else {
      long lo, hi;
      chunk_range(n, conn_chunks, i - nblocks, lo, hi);
      char ln[256];
      for (long c = lo; c < hi; c++) {
        const int32_t* v = cell_vertices + 8 * c;
        std::snprintf(ln, sizeof ln, "%d %d %d %d %d %d %d %d\n ", v[0] + 1, v[1] + 1, v[2] + 1, v[3] + 1,
                      v[4] + 1, v[5] + 1, v[6] + 1, v[7] + 1);
        o += ln;
      }
    }
  });
  size_t total = out.size();
  for (auto& p : parts) total += p.size();
  out.reserve(total);
  for (auto& p : parts) out += p;
  return out;
}

std::string grid_text(const HostCase& hc) {
  std::string out = "title = \"cycas partition grid\"\nvariables=\"x\",\"y\",\"z\",\"p\"\n";
  char line[512];
  std::snprintf(line, sizeof line, "zone n=%d, e=%d, f=fepoint, et=BRICK\n", hc.nvrt, hc.ncel);
  out += line;
  // the fourth value marks vertices on a partition interface: none with one partition
  for (int i = 0; i < hc.nvrt; i++) {
    const double* x = &hc.vert[3 * (size_t)i];
    std::snprintf(line, sizeof line, "%f %f %f %f\n", x[0], x[1], x[2], 0.0);
    out += line;
  }
  for (int i = 0; i < hc.ncel; i++) {
    const int32_t* v = &hc.cell_vertices[8 * (size_t)i];
    std::snprintf(line, sizeof line, "%8d %8d %8d %8d %8d %8d %8d %8d\n", v[0] + 1, v[1] + 1, v[2] + 1, v[3] + 1,
                  v[4] + 1, v[5] + 1, v[6] + 1, v[7] + 1);
    out += line;
  }
  return out;
}

std::string geo_bytes(const HostCase& hc) {
  std::string out;
  out.reserve(16 + 24 * (size_t)hc.nvrt + 32 * (size_t)hc.ncel);
  append_i32(out, 0);  // rank
  append_i32(out, 1);  // number of partitions
  append_i32(out, hc.ncel);
  append_i32(out, hc.nvrt);
  append_f64(out, hc.vert.data(), 3L * hc.nvrt);
  for (size_t i = 0; i < 8 * (size_t)hc.ncel; i++) append_i32(out, hc.cell_vertices[i] + 1);
  return out;
}

std::string data_bytes(const CellFieldsView& f) {
  const int nvar = f.turb == 1 ? 8 : 6;
  std::string out;
  out.reserve(8 + sizeof(double) * (size_t)nvar * (size_t)f.ncel);
  append_i32(out, 0);
  append_i32(out, nvar);
  for (const double* a : {f.P, f.U, f.V, f.W, f.R, f.T}) append_f64(out, a, f.ncel);
  if (f.turb == 1) {
    append_f64(out, f.TE, f.ncel);
    append_f64(out, f.ED, f.ncel);
  }
  return out;
}

// ostream's default double conversion is printf's %g (six significant digits)
std::string backup_text(const CellFieldsView& f) {
  const int chunks = 64;
  std::vector<std::string> parts = render_parts(chunks, [&](int ch, std::string& out) {
    long lo, hi;
    chunk_range(f.ncel, chunks, ch, lo, hi);
    char line[512];
    for (long i = lo; i < hi; i++) {
      std::snprintf(line, sizeof line, "%g %g %g %g %g %g %g %g\n", f.R[i], f.U[i], f.V[i], f.W[i], f.P[i],
                    f.T[i], f.R[i], f.VisLam[i]);
      out += line;
      if (f.turb == 1) {
        std::snprintf(line, sizeof line, "%g %g %g\n", f.VisTur[i], f.TE[i], f.ED[i]);
        out += line;
      }
    }
  });
  std::string out;
  size_t total = 0;
  for (auto& p : parts) total += p.size();
  out.reserve(total);
  for (auto& p : parts) out += p;
  return out;
}

void read_backup(const std::string& path, long ncel, int turb, double* const out[10]) {
  FILE* fp = std::fopen(path.c_str(), "rb");
  if (!fp) throw IoError("cannot open backup file " + path);
  std::string text;
  char buf[1 << 16];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof buf, fp)) > 0) text.append(buf, got);
  std::fclose(fp);
  const char* p = text.c_str();
  auto next = [&](long cell) {
    char* end = nullptr;
    errno = 0;
    double v = std::strtod(p, &end);
    if (end == p) throw IoError(path + ": too few values (cell " + std::to_string(cell) + ")");
    p = end;
    return v;
  };
  // ReadBackupFile order: R U V W P T R VisLam [VisTur TE ED]; the second R is the one kept
  const int order[8] = {0, 1, 2, 3, 4, 5, 0, 6};
  for (long i = 0; i < ncel; i++) {
    for (int k = 0; k < 8; k++) out[order[k]][i] = next(i);
    if (turb == 1)
      for (int k = 7; k < 10; k++) out[k][i] = next(i);
  }
}

void write_file(const std::string& path, const std::string& bytes) {
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) throw IoError("cannot open " + path + " for writing: " + std::strerror(errno));
  size_t put = std::fwrite(bytes.data(), 1, bytes.size(), fp);
  int rc = std::fclose(fp);
  if (put != bytes.size() || rc != 0) throw IoError("short write to " + path);
}

}  // namespace cycas
