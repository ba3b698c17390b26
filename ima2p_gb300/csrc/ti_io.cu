// ti_io.cu -- saved-genealogy (.ti) files for the L-mode surface: the
// reference's text format (loadgenealogyvalues, ima_main_mpi.cpp:3216-3440;
// savegenealogyfile, output.cpp:662-685) read straight into the resident
// gsampinf rows, and a binary side-car that reloads without parsing.
//
// Text: header lines up to one containing "VALUESSTART", then one line per
// genealogy of `rowlen` values (written "%.6f\t", read as float).  When more
// genealogies are present than are to be loaded, the reference keeps a line
// while loaded / (loaded + notloaded) <= numtoload / total, counting across
// the files in the order given; the same rule is applied here to the line
// indices before any value is parsed, and the kept lines are parsed by all
// host threads.
#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "ima_gpu.h"

namespace {

constexpr int MAXGENEALOGIESTOSAVE = 300000;  // imamp.hpp:149

struct TiFile {
  std::string text;
  size_t values_begin = 0;          // first byte after the VALUESSTART line
  std::vector<size_t> line_begin;   // genealogy lines
};

bool read_file(const char *path, std::string *out)
{
  FILE *f = fopen(path, "rb");
  if (!f) return false;
  fseek(f, 0, SEEK_END);
  long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  out->resize(n > 0 ? (size_t)n : 0);
  size_t got = n > 0 ? fread(&(*out)[0], 1, (size_t)n, f) : 0;
  fclose(f);
  return got == out->size();
}

// the genealogy lines: every '\n'-terminated line after the VALUESSTART line
// (the reference counts newlines there)
bool index_lines(TiFile *t)
{
  const std::string &s = t->text;
  size_t pos = 0;
  bool found = false;
  while (pos < s.size()) {
    size_t e = s.find('\n', pos);
    if (e == std::string::npos) e = s.size();
    const size_t v = s.find("VALUESSTART", pos);
    if (v != std::string::npos && v < e) {
      found = true;
      pos = e + 1;
      break;
    }
    pos = e + 1;
  }
  if (!found) return false;
  t->values_begin = pos;
  while (pos < s.size()) {
    size_t e = s.find('\n', pos);
    if (e == std::string::npos) break;  // an unterminated last line is not counted
    t->line_begin.push_back(pos);
    pos = e + 1;
  }
  return true;
}

// parses exactly rowlen values from the line at p; false on too few or too many
bool parse_line(const char *p, const char *end, int rowlen, float *row)
{
  for (int i = 0; i < rowlen; i++) {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) p++;
    if (p >= end || *p == '\n') return false;
    char *q = nullptr;
    row[i] = strtof(p, &q);  // correctly rounded, as sscanf("%f") rounds
    if (q == p) return false;
    p = q;
  }
  while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) p++;
  return p >= end || *p == '\n';
}

}  // namespace

extern "C" int ima_ti_read(int nfiles, const char *const *paths, int rowlen, int maxload, float *rows,
                           int rows_cap, int *loaded, int *total)
{
  if (nfiles < 1 || !paths || rowlen < 1 || !loaded || !total) return IMA_ERR_ARG;
  std::vector<TiFile> files(nfiles);
  long long tot = 0;
  for (int f = 0; f < nfiles; f++) {
    if (!paths[f] || !read_file(paths[f], &files[f].text)) return IMA_ERR_ARG;
    if (!index_lines(&files[f])) return IMA_ERR_DATA;
    tot += (long long)files[f].line_begin.size();
  }
  if (tot < 1) return IMA_ERR_DATA;
  long long numtoload = tot;
  if (maxload > 0) numtoload = std::min<long long>(numtoload, maxload);
  numtoload = std::min<long long>(numtoload, MAXGENEALOGIESTOSAVE);
  const bool loadall = numtoload >= tot;
  const float load_fraction = (float)numtoload / (float)tot;
  // which lines the reference keeps, in file order
  std::vector<std::pair<int, size_t>> keep;  // (file, line)
  long long nl = 0, nn = 0;
  for (int f = 0; f < nfiles; f++)
    for (size_t l = 0; l < files[f].line_begin.size(); l++) {
      if (loadall || nl == 0 || ((float)nl / (float)(nl + nn)) <= load_fraction) {
        keep.push_back({f, l});
        nl++;
      } else {
        nn++;
      }
    }
  *total = (int)tot;
  *loaded = (int)keep.size();
  if (!rows) return IMA_OK;  // a count only
  if ((int)keep.size() > rows_cap) return IMA_ERR_TOO_LARGE;
  // parse the kept lines on every host thread
  const int nth = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  std::vector<int> bad(nth, -1);
  std::vector<std::thread> th;
  for (int t = 0; t < nth; t++)
    th.emplace_back([&, t] {
      for (size_t k = t; k < keep.size(); k += nth) {
        const TiFile &tf = files[keep[k].first];
        const size_t b = tf.line_begin[keep[k].second];
        const char *p = tf.text.data() + b, *end = tf.text.data() + tf.text.size();
        if (!parse_line(p, end, rowlen, rows + k * (size_t)rowlen)) {
          bad[t] = (int)k;
          return;
        }
      }
    });
  for (auto &x : th) x.join();
  for (int t = 0; t < nth; t++)
    if (bad[t] >= 0) return IMA_ERR_DATA;  // too few or too many values on a line
  return IMA_OK;
}

// binary side-car: magic, rowlen, G, then G * rowlen floats (little endian)
static const char TI_MAGIC[8] = {'I', 'M', 'A', 'T', 'I', 'B', '0', '1'};

extern "C" int ima_ti_write_binary(const char *path, int G, int rowlen, const float *rows)
{
  if (!path || G < 0 || rowlen < 1 || (G > 0 && !rows)) return IMA_ERR_ARG;
  FILE *f = fopen(path, "wb");
  if (!f) return IMA_ERR_ARG;
  int32_t hdr[2] = {rowlen, G};
  bool ok = fwrite(TI_MAGIC, 1, 8, f) == 8 && fwrite(hdr, 4, 2, f) == 2 &&
            fwrite(rows, sizeof(float), (size_t)G * rowlen, f) == (size_t)G * rowlen;
  ok = (fclose(f) == 0) && ok;
  return ok ? IMA_OK : IMA_ERR_DATA;
}

extern "C" int ima_ti_read_binary(const char *path, int *G, int *rowlen, float *rows, int rows_cap)
{
  if (!path || !G || !rowlen) return IMA_ERR_ARG;
  FILE *f = fopen(path, "rb");
  if (!f) return IMA_ERR_ARG;
  char magic[8];
  int32_t hdr[2];
  if (fread(magic, 1, 8, f) != 8 || memcmp(magic, TI_MAGIC, 8) != 0 || fread(hdr, 4, 2, f) != 2 || hdr[0] < 1 ||
      hdr[1] < 0) {
    fclose(f);
    return IMA_ERR_DATA;
  }
  int r = IMA_OK;
  if (rows) {
    // *rowlen on input: the row length the caller sized rows for; the file
    // may have changed since the header call
    if (hdr[0] != *rowlen) r = IMA_ERR_DATA;
    else if (rows_cap < 0 || hdr[1] > rows_cap) r = IMA_ERR_TOO_LARGE;
    else if (fread(rows, sizeof(float), (size_t)hdr[0] * hdr[1], f) != (size_t)hdr[0] * hdr[1]) r = IMA_ERR_DATA;
  }
  *rowlen = hdr[0];
  *G = hdr[1];
  fclose(f);
  return r;
}
