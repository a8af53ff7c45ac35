/*
 * plt_writer.cpp -- host half of the snapshot writers (see plt_writer.h).
 * Byte layout of the particle file header, as MPM::Output_plt_file writes it
 * through Write_file (glbfunc.h:302-305: every value in its own size, so ints
 * are 4 bytes and the marker floats 4, the time and ranges 8; names one int32
 * per character and a 0).
 */
#include "plt_writer.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

namespace pgdg_out {

namespace {
template <class T>
void put(std::string& s, T v) {
  char b[sizeof(T)];
  std::memcpy(b, &v, sizeof(T));
  s.append(b, sizeof(T));
}
void put_name(std::string& s, const char* name) {
  for (const char* c = name; *c; c++) put<int32_t>(s, (int32_t)(unsigned char)*c);
  put<int32_t>(s, 0);
}
}  // namespace

std::string plt_header(int64_t n, double time) {
  static const char* names[12] = {"x", "y", "z", "phase", "vx", "vy", "vol", "rho", "P", "tv", "v", "n_neighbor"};
  static const int32_t types[12] = {2, 2, 2, 3, 2, 2, 2, 2, 2, 2, 2, 3}; /* 2 double, 3 int32 */
  std::string s;
  s.append("#!TDV112", 8);
  put<int32_t>(s, 1);  /* byte order */
  put<int32_t>(s, 0);  /* file type: full */
  put<int32_t>(s, 0);  /* title: empty */
  put<int32_t>(s, 12);
  for (auto nm : names) put_name(s, nm);
  put<float>(s, 299.0f); /* zone marker */
  put_name(s, "grid");
  put<int32_t>(s, -1);   /* parent zone */
  put<int32_t>(s, 0);    /* strand */
  put<double>(s, time);  /* solution time */
  put<int32_t>(s, -1);   /* zone colour */
  put<int32_t>(s, 0);    /* ordered zone */
  put<int32_t>(s, 0);    /* no variable location */
  put<int32_t>(s, 0);    /* no face neighbours */
  put<int32_t>(s, 0);    /* no miscellaneous connectivity */
  put<int32_t>(s, (int32_t)n);
  put<int32_t>(s, 1);
  put<int32_t>(s, 1);
  put<int32_t>(s, 0);    /* no auxiliary data */
  put<float>(s, 357.0f); /* end of header */
  put<float>(s, 299.0f); /* zone data */
  for (auto t : types) put<int32_t>(s, t);
  put<int32_t>(s, 0);    /* no passive variables */
  put<int32_t>(s, 0);    /* no variable sharing */
  put<int32_t>(s, -1);   /* no connectivity sharing */
  for (int j = 0; j < 12; j++) {
    put<double>(s, -1.0);
    put<double>(s, 1.0);
  }
  return s;
}

int write_cell_table(const char* path, int dim, const int N[3], const double box_l[3], const double p_size[3],
                     const double* cols, double time, int threads, std::string* msg) {
  FILE* f = std::fopen(path, "w");
  if (!f) {
    if (msg) *msg = std::string("cannot open ") + path;
    return -1;
  }
  char tb[64];
  std::snprintf(tb, sizeof(tb), "%g", time);
  std::string head = "VARIABLES = \"x\",\"y\",\"z\", \"v1\",\"v2\", \"v\",\"rho0\",\"rho1\",        "
                     "\"E0\",\"E1\",\"Lim0\",\"Lim1\",\"st\", \"st1\", \"P\"\n";
  head += std::string("ZONE T=\"GRID 1\",SOLUTIONTIME=") + tb + "\n";
  bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size();
  const int64_t nz = dim == 3 ? N[2] : 1;
  const int64_t ncell = (int64_t)N[0] * N[1] * nz;
  const int64_t chunk = 1 << 16;
  const int nt = std::max(1, threads);
  std::vector<std::string> bufs(nt);
  /* rounds of nt chunks: formatted in parallel, written in order */
  for (int64_t c0 = 0; c0 < ncell && ok; c0 += chunk * nt) {
    std::vector<std::thread> ths;
    for (int w = 0; w < nt; w++) {
      ths.emplace_back([&, w] {
        std::string& out = bufs[w];
        out.clear();
        const int64_t a = c0 + w * chunk, b = std::min(ncell, a + chunk);
        char line[512];
        for (int64_t ci = a; ci < b; ci++) {
          const int64_t i = ci / ((int64_t)N[1] * nz), j = (ci / nz) % N[1], k = ci % nz;
          const double x = box_l[0] + p_size[0] * (i + 0.5), y = box_l[1] + p_size[1] * (j + 0.5);
          const double z = dim == 3 ? box_l[2] + p_size[2] * (k + 0.5) : 0.0;
          const double* o = cols + 12 * ci;
          const int len = std::snprintf(line, sizeof(line), "%g %g %g %g %g %g %g %g %g %g %g %g %g %g %g \n", x, y, z,
                                        o[0], o[1], o[2], o[3], o[4], o[5], o[6], o[7], o[8], o[9], o[10], o[11]);
          out.append(line, (size_t)std::min<int>(len, (int)sizeof(line) - 1));
        }
      });
    }
    for (auto& t : ths) t.join();
    for (int w = 0; w < nt && ok; w++) ok = std::fwrite(bufs[w].data(), 1, bufs[w].size(), f) == bufs[w].size();
  }
  if (std::fclose(f) != 0) ok = false;
  if (!ok) {
    if (msg) *msg = std::string("write failed: ") + path;
    return -1;
  }
  return 0;
}

}  // namespace pgdg_out
