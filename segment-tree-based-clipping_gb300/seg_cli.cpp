// seg -- drop-in replacement of the reference's `bin/seg` driver
// (src/clip.cpp:2117-2130 main -> multicore_clipping :1415), running the
// clipping on the GPU through libsbclip.so.
//
//   seg <base> <overlay_1> [<overlay_2> ... <overlay_k>] [--out DIR] [--precision P]
//       [--device D] [--union]
//
// Input files: the vertex count, then one `x,y` (or `x y`) line per vertex,
// no closing duplicate (src/clip.cpp:181-298).  For overlay i the rings of
// base ∩ overlay_i are written to DIR/Fig-def-R<i>.txt (default DIR
// ../results, src/clip.cpp:31-32 and :2048-2051), `x y,` per vertex and `;`
// per ring at ostream precision P (default 6, foster/polygon.h:576-585).
// The `README.md` form `seg <base> <overlay> <result path>` is accepted when
// the third argument is not a readable polygon file: it names the output
// file.  With one overlay, the larger polygon is the base (the reference's
// pairwise reader, src/clip.cpp:63-77; its copy loop requires it).  stdout:
// a banner, `R ` per overlay, then the reference's TIME line fields in
// microseconds: skeleton endlist cover cand+merge label total.  --union
// writes base ∪ overlay_i instead (the Foster back end's UNION switch,
// foster/polyclip.h:39, which the reference's driver leaves off).
//
//   seg <P.poly> <Q.poly> <R.poly> [--union]
//
// Polygons with several components (holes, islands) in the .poly format of
// the reference's Foster program (lib/optimizedFostersAlgorithm/README.md:
// 43-62: `x y,` per vertex, `;` closing each component, no count line) are
// clipped as such (sbc_clip_components), P as the base, and R written in the
// same format.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sbclip.h"

namespace {

bool read_poly(const char* path, std::vector<double>& xy) {
  FILE* f = fopen(path, "r");
  if (!f) return false;
  int n = 0;
  if (fscanf(f, "%d", &n) != 1 || n < 0) {
    fclose(f);
    return false;
  }
  xy.resize(2 * (size_t)n);
  for (int i = 0; i < n; ++i) {
    double x, y;
    // `%lf,%lf` as the reference; also `x y`
    if (fscanf(f, " %lf", &x) != 1) {
      fclose(f);
      return false;
    }
    int c = fgetc(f);
    while (c == ' ' || c == '\t') c = fgetc(f);
    if (c != ',') ungetc(c, f);
    if (fscanf(f, " %lf", &y) != 1) {
      fclose(f);
      return false;
    }
    xy[2 * i] = x;
    xy[2 * i + 1] = y;
  }
  fclose(f);
  return true;
}

// Foster's .poly format: the first line holds a vertex (two numbers), not a
// vertex count
bool is_foster_file(const char* path) {
  FILE* f = fopen(path, "r");
  if (!f) return false;
  double x, y;
  bool ok = fscanf(f, " %lf %lf", &x, &y) == 2;
  if (ok) {
    int c = fgetc(f);
    while (c == ' ' || c == '\t') c = fgetc(f);
    ok = c == ',' || c == ';';
  }
  fclose(f);
  return ok;
}

// polygon.h operator>> (foster/polygon.h:550-571) per component: `x y`
// then `,` (more vertices) or `;` (component ends); comp receives the
// component starts and the vertex count
bool read_foster(const char* path, std::vector<double>& xy, std::vector<int>& comp) {
  FILE* f = fopen(path, "r");
  if (!f) return false;
  xy.clear();
  comp.assign(1, 0);
  double x, y;
  int n = 0;
  while (fscanf(f, " %lf %lf", &x, &y) == 2) {
    xy.push_back(x);
    xy.push_back(y);
    ++n;
    int c = fgetc(f);
    while (c == ' ' || c == '\t') c = fgetc(f);
    if (c != ',') comp.push_back(n);  // `;`, a line end or the end of the file
    if (c == EOF) break;
  }
  if (comp.back() != n) comp.push_back(n);
  fclose(f);
  return n > 0;
}

bool is_poly_file(const char* path) {
  FILE* f = fopen(path, "r");
  if (!f) return false;
  int n;
  bool ok = fscanf(f, "%d", &n) == 1;
  fclose(f);
  return ok;
}

bool write_rings(const std::string& path, const sbc_rings& r, int precision) {
  FILE* f = fopen(path.c_str(), "w");
  if (!f) return false;
  char fmt[32];
  snprintf(fmt, sizeof fmt, "%%.%dg %%.%dg", precision, precision);
  for (int j = 0; j < r.nrings; ++j) {
    for (int v = r.offsets[j]; v < r.offsets[j + 1]; ++v) {
      fprintf(f, fmt, r.xy[2 * v], r.xy[2 * v + 1]);
      fputs(v + 1 < r.offsets[j + 1] ? ",\n" : ";\n", f);
    }
  }
  fclose(f);
  return true;
}

}  // namespace

int main(int argc, char** argv) {
  std::vector<const char*> pos;
  std::string outdir = "../results", outfile;
  int precision = 6, device = 0, flags = SBC_FLAG_TIMING;
  for (int i = 1; i < argc; ++i) {
    if (!strcmp(argv[i], "--out") && i + 1 < argc) outdir = argv[++i];
    else if (!strcmp(argv[i], "--precision") && i + 1 < argc) precision = atoi(argv[++i]);
    else if (!strcmp(argv[i], "--device") && i + 1 < argc) device = atoi(argv[++i]);
    else if (!strcmp(argv[i], "--union")) flags |= SBC_FLAG_UNION;
    else pos.push_back(argv[i]);
  }
  if (pos.size() < 2) {
    printf("3 parameters required\n./seg <base polygon path> <subject polygon path>\n");
    return 1;
  }
  if (pos.size() == 3 && is_foster_file(pos[0]) && is_foster_file(pos[1])) {
    std::vector<double> pxy, qxy;
    std::vector<int> pk, qk;
    if (!read_foster(pos[0], pxy, pk) || !read_foster(pos[1], qxy, qk)) {
      fprintf(stderr, "cannot read the .poly inputs\n");
      return 1;
    }
    sbc_options opt{device, flags};
    sbc_ctx* ctx = nullptr;
    if (sbc_create(&opt, &ctx)) {
      fprintf(stderr, "sbc_create failed\n");
      return 2;
    }
    sbc_rings r;
    int rc = sbc_clip_components(ctx, pxy.data(), pk.data(), (int)pk.size() - 1, qxy.data(),
                                 qk.data(), (int)qk.size() - 1, &r, nullptr);
    if (rc) {
      fprintf(stderr, "clipping failed (%d): %s\n", rc, sbc_last_error(ctx));
      sbc_destroy(ctx);
      return 3;
    }
    if (!write_rings(pos[2], r, precision)) fprintf(stderr, "cannot write %s\n", pos[2]);
    printf("R %d rings\n", r.nrings);
    sbc_destroy(ctx);
    return 0;
  }
  if (pos.size() == 3 && !is_poly_file(pos[2])) {
    outfile = pos[2];
    pos.pop_back();
  }
  std::vector<double> b;
  if (!read_poly(pos[0], b)) {
    fprintf(stderr, "cannot read base polygon %s\n", pos[0]);
    return 1;
  }
  std::vector<double> c;
  std::vector<int> sizes;
  for (size_t i = 1; i < pos.size(); ++i) {
    std::vector<double> o;
    if (!read_poly(pos[i], o)) {
      fprintf(stderr, "cannot read overlay polygon %s\n", pos[i]);
      return 1;
    }
    sizes.push_back((int)(o.size() / 2));
    c.insert(c.end(), o.begin(), o.end());
  }
  if (sizes.size() == 1 && (int)(b.size() / 2) < sizes[0]) {
    b.swap(c);
    sizes[0] = (int)(c.size() / 2);
  }
  printf("GB300 algorithm\n");
  sbc_options opt{device, flags};
  sbc_ctx* ctx = nullptr;
  int rc = sbc_create(&opt, &ctx);
  if (rc) {
    fprintf(stderr, "sbc_create failed (%d)\n", rc);
    return 2;
  }
  std::vector<sbc_rings> out(sizes.size());
  auto t0 = std::chrono::high_resolution_clock::now();
  rc = sbc_clip_one_to_many(ctx, b.data(), (int)(b.size() / 2), c.data(), sizes.data(),
                            (int)sizes.size(), out.data(), nullptr);
  auto t1 = std::chrono::high_resolution_clock::now();
  if (rc) {
    fprintf(stderr, "clipping failed (%d): %s\n", rc, sbc_last_error(ctx));
    sbc_destroy(ctx);
    return 3;
  }
  for (size_t i = 0; i < out.size(); ++i) {
    printf("R ");
    std::string path = outfile.empty() ? outdir + "/Fig-def-R" + std::to_string(i + 1) + ".txt"
                                       : outfile;
    if (!write_rings(path, out[i], precision)) fprintf(stderr, "cannot write %s\n", path.c_str());
  }
  float ms[8];
  sbc_phase_times(ctx, ms, 8);
  long long total = std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count();
  printf(" %lld %lld %lld %lld %lld %lld\n", (long long)((ms[0] + ms[1]) * 1000),
         (long long)(ms[2] * 1000), (long long)(ms[3] * 1000), (long long)(ms[4] * 1000),
         (long long)((ms[5] + ms[6]) * 1000), total);
  sbc_destroy(ctx);
  return 0;
}
