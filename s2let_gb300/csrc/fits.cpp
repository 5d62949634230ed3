// FITS I/O of MW / MWSS maps: the reference's s2let_fits entry points
// (include/s2let/s2let_fits.h:18-106, src/c/s2let_fits.c:17-551) without
// cfitsio.  The files are what cfitsio writes there: an empty primary HDU
// (BITPIX 16, NAXIS 0, EXTEND) and one binary-table extension named BINTABLE
// with one double column SIGNAL (or Q_POLARISATION and U_POLARISATION), one
// sample per row, and the keywords L (and MWSS = 1 for MWSS maps).  The reader
// takes any binary table whose first (second) column is of type D (8-byte
// float) or E (4-byte float) with any repeat count, read as one stream in row
// order, as cfitsio's fits_read_col does.
//
// Format (FITS standard 4.0): 2880-byte blocks; header units of 80-character
// ASCII cards "KEYWORD = value / comment" ending with END, padded with spaces;
// binary table data big-endian, padded with zeros.
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "host_layer.h"
#include "runtime.h"

namespace s2g {
namespace {

constexpr size_t kBlock = 2880;

// ---- writing ----------------------------------------------------------------

std::string pad80(std::string c) {
  c.resize(80, ' ');
  return c;
}
std::string card_value(const char *key, const std::string &value, const char *comment) {
  char buf[96];
  snprintf(buf, sizeof buf, "%-8.8s= %20s / %s", key, value.c_str(), comment);
  return pad80(buf);
}
std::string card_string(const char *key, const char *s, const char *comment) {
  std::string q = std::string("'") + s;
  while (q.size() < 9) q.push_back(' ');  // strings are padded to 8 characters
  q.push_back('\'');
  char buf[96];
  snprintf(buf, sizeof buf, "%-8.8s= %-20s / %s", key, q.c_str(), comment);
  return pad80(buf);
}
void pad_block(std::string &h, char fill) {
  while (h.size() % kBlock) h.push_back(fill);
}
void put_be64(std::string &out, double v) {
  uint64_t u;
  memcpy(&u, &v, 8);
  for (int i = 7; i >= 0; --i) out.push_back((char)((u >> (8 * i)) & 0xFF));
}

// cfitsio refuses an existing file unless the name starts with '!'
void write_table(const char *name, int L, bool mwss, const std::vector<std::pair<const char *, const double *>> &cols,
                 int64_t npix) {
  S2G_REQUIRE(name != nullptr && name[0] != 0, ERR_INVALID, "NULL file name");
  std::string path = name;
  bool clobber = false;
  if (path[0] == '!') {
    clobber = true;
    path = path.substr(1);
  }
  if (!clobber) {
    FILE *t = fopen(path.c_str(), "rb");
    if (t) {
      fclose(t);
      S2G_REQUIRE(false, ERR_INVALID, "Could not create new fits file (it exists; prefix the name with '!')");
    }
  }
  std::string h;
  h += card_value("SIMPLE", "T", "file does conform to FITS standard");
  h += card_value("BITPIX", "16", "number of bits per data pixel");
  h += card_value("NAXIS", "0", "number of data axes");
  h += card_value("EXTEND", "T", "FITS dataset may contain extensions");
  h += pad80("END");
  pad_block(h, ' ');
  const int nf = (int)cols.size();
  h += card_string("XTENSION", "BINTABLE", "binary table extension");
  h += card_value("BITPIX", "8", "8-bit bytes");
  h += card_value("NAXIS", "2", "2-dimensional binary table");
  h += card_value("NAXIS1", std::to_string(8 * nf), "width of table in bytes");
  h += card_value("NAXIS2", std::to_string(npix), "number of rows in table");
  h += card_value("PCOUNT", "0", "size of special data area");
  h += card_value("GCOUNT", "1", "one data group (required keyword)");
  h += card_value("TFIELDS", std::to_string(nf), "number of fields in each row");
  for (int c = 0; c < nf; ++c) {
    const std::string k = std::to_string(c + 1);
    h += card_string(("TTYPE" + k).c_str(), cols[c].first, ("label for field " + k).c_str());
    h += card_string(("TFORM" + k).c_str(), "1D", "data format of field: 8-byte DOUBLE");
    h += card_string(("TUNIT" + k).c_str(), " ", "physical unit of field");
  }
  h += card_string("EXTNAME", "BINTABLE", "name of this binary table extension");
  h += card_value("L", std::to_string(L), "Resolution parameter");
  if (mwss) h += card_value("MWSS", "1", "Sampling scheme parameter");
  h += pad80("END");
  pad_block(h, ' ');
  std::string d;
  d.reserve((size_t)npix * 8 * nf + kBlock);
  for (int64_t i = 0; i < npix; ++i)
    for (int c = 0; c < nf; ++c) put_be64(d, cols[c].second[i]);
  pad_block(d, '\0');
  FILE *fp = fopen(path.c_str(), "wb");
  S2G_REQUIRE(fp != nullptr, ERR_INVALID, "Could not create new fits file");
  const bool ok = fwrite(h.data(), 1, h.size(), fp) == h.size() && fwrite(d.data(), 1, d.size(), fp) == d.size();
  fclose(fp);
  S2G_REQUIRE(ok, ERR_INVALID, "Could not write signal");
}

// ---- reading ----------------------------------------------------------------

struct Hdu {
  std::map<std::string, std::string> keys;  // keyword -> value field (trimmed, quotes removed)
  size_t data_offset = 0;
};

std::string trim(const std::string &s) {
  size_t a = s.find_first_not_of(' '), b = s.find_last_not_of(' ');
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

// parses the header starting at `pos`; returns false on a malformed file
bool parse_header(const std::vector<char> &buf, size_t &pos, Hdu &h) {
  for (;;) {
    if (pos + kBlock > buf.size()) return false;
    bool end = false;
    for (size_t i = 0; i < kBlock; i += 80) {
      const std::string c(&buf[pos + i], 80);
      const std::string key = trim(c.substr(0, 8));
      if (key == "END") {
        end = true;
        break;
      }
      if (c.size() > 9 && c[8] == '=' && c[9] == ' ') {
        std::string v = c.substr(10);
        if (!v.empty() && trim(v)[0] == '\'') {  // string value, '' escapes a quote
          std::string t = trim(v).substr(1), out;
          for (size_t k = 0; k < t.size(); ++k) {
            if (t[k] == '\'') {
              if (k + 1 < t.size() && t[k + 1] == '\'') {
                out.push_back('\'');
                ++k;
                continue;
              }
              break;
            }
            out.push_back(t[k]);
          }
          v = trim(out);
        } else {
          const size_t sl = v.find('/');
          if (sl != std::string::npos) v = v.substr(0, sl);
          v = trim(v);
        }
        h.keys[key] = v;
      }
    }
    pos += kBlock;
    if (end) break;
  }
  h.data_offset = pos;
  return true;
}

long key_long(const Hdu &h, const char *k, bool *found) {
  auto it = h.keys.find(k);
  *found = it != h.keys.end();
  return *found ? atol(it->second.c_str()) : 0;
}

// the second HDU (first extension) of a file; throws when absent or not a binary table
Hdu open_table(const char *name, std::vector<char> &buf) {
  S2G_REQUIRE(name != nullptr, ERR_INVALID, "NULL file name");
  FILE *fp = fopen(name, "rb");
  S2G_REQUIRE(fp != nullptr, ERR_INVALID, std::string("could not open FITS file ") + name);
  fseek(fp, 0, SEEK_END);
  const long n = ftell(fp);
  fseek(fp, 0, SEEK_SET);
  buf.resize(n > 0 ? (size_t)n : 0);
  const size_t got = n > 0 ? fread(buf.data(), 1, (size_t)n, fp) : 0;
  fclose(fp);
  S2G_REQUIRE(got == buf.size(), ERR_INVALID, "could not read FITS file");
  Hdu prim, ext;
  size_t pos = 0;
  S2G_REQUIRE(parse_header(buf, pos, prim), ERR_INVALID, "malformed FITS primary header");
  // skip the primary data unit
  bool f;
  const long naxis = key_long(prim, "NAXIS", &f), bitpix = key_long(prim, "BITPIX", &f);
  size_t nbytes = 0;
  if (naxis > 0) {
    nbytes = (size_t)(bitpix < 0 ? -bitpix : bitpix) / 8;
    for (long i = 1; i <= naxis; ++i) nbytes *= (size_t)key_long(prim, ("NAXIS" + std::to_string(i)).c_str(), &f);
  }
  pos += (nbytes + kBlock - 1) / kBlock * kBlock;
  S2G_REQUIRE(parse_header(buf, pos, ext), ERR_INVALID, "the FITS file has no extension (HDU 2)");
  if (ext.keys["XTENSION"] != "BINTABLE") fprintf(stderr, "%s: Extension is not binary!\n", __FILE__);
  return ext;
}

// column `col` (1-based) of the binary table as one stream of doubles (row order)
std::vector<double> read_column(const std::vector<char> &buf, const Hdu &h, int col) {
  bool f1, f2, f3;
  const long row = key_long(h, "NAXIS1", &f1), nrows = key_long(h, "NAXIS2", &f2), nf = key_long(h, "TFIELDS", &f3);
  S2G_REQUIRE(f1 && f2 && f3 && col >= 1 && col <= nf, ERR_INVALID, "binary table without the requested column");
  S2G_REQUIRE(row > 0 && nrows >= 0, ERR_INVALID, "binary table with a bad NAXIS1 / NAXIS2");
  size_t off = 0;
  long rep = 0;
  char type = 0;
  for (int c = 1; c <= col; ++c) {
    auto it = h.keys.find("TFORM" + std::to_string(c));
    S2G_REQUIRE(it != h.keys.end(), ERR_INVALID, "binary table column without TFORM");
    const std::string t = it->second;
    size_t k = 0;
    while (k < t.size() && isdigit((unsigned char)t[k])) ++k;
    const long r = k ? atol(t.substr(0, k).c_str()) : 1;
    const char ty = k < t.size() ? t[k] : 0;
    static const std::map<char, int> width = {{'L', 1}, {'X', 0}, {'B', 1}, {'I', 2}, {'J', 4}, {'K', 8},
                                              {'A', 1}, {'E', 4}, {'D', 8}, {'C', 8}, {'M', 16}};
    auto w = width.find(ty);
    S2G_REQUIRE(w != width.end(), ERR_INVALID, "unsupported binary table column type");
    if (c < col) {
      off += ty == 'X' ? (size_t)(r + 7) / 8 : (size_t)r * w->second;
    } else {
      rep = r;
      type = ty;
    }
  }
  S2G_REQUIRE(type == 'D' || type == 'E', ERR_INVALID, "map column is neither 8-byte (D) nor 4-byte (E) float");
  // the column must lie inside one row, and the rows inside the file
  S2G_REQUIRE(rep >= 0 && off + (size_t)rep * (type == 'D' ? 8 : 4) <= (size_t)row, ERR_INVALID,
              "binary table column extends past the end of its row (TFORMs wider than NAXIS1)");
  const size_t need = h.data_offset + (size_t)row * nrows;
  S2G_REQUIRE(need <= buf.size(), ERR_INVALID, "truncated FITS data unit");
  std::vector<double> out;
  out.reserve((size_t)nrows * rep);
  for (long r = 0; r < nrows; ++r) {
    const unsigned char *p = (const unsigned char *)&buf[h.data_offset + (size_t)r * row + off];
    for (long e = 0; e < rep; ++e) {
      if (type == 'D') {
        uint64_t u = 0;
        for (int i = 0; i < 8; ++i) u = (u << 8) | p[8 * e + i];
        double v;
        memcpy(&v, &u, 8);
        out.push_back(v);
      } else {
        uint32_t u = 0;
        for (int i = 0; i < 4; ++i) u = (u << 8) | p[4 * e + i];
        float v;
        memcpy(&v, &u, 4);
        out.push_back((double)v);
      }
    }
  }
  return out;
}

// src/c/s2let_fits.c:177-234 (MW) and 236-300 (MWSS); ncol 1 (map) or 2 (Q, U)
void read_maps(double *const *dst, int ncol, const char *name, int L, bool mwss, bool spin_prints) {
  S2G_REQUIRE(L >= 1, ERR_INVALID, "L must be >= 1");
  std::vector<char> buf;
  Hdu h = open_table(name, buf);
  bool f;
  const long Lread = key_long(h, "L", &f);
  S2G_REQUIRE(f, ERR_INVALID, "keyword L not found");
  if (Lread != L) printf("Attention : read L = %li but you specified L = %i\n", Lread, L);
  if (mwss) {
    const long m = key_long(h, "MWSS", &f);
    S2G_REQUIRE(f, ERR_INVALID, "keyword MWSS not found");
    if (m != 1) printf("Attention : the file is not stored with MWSS sampling.\n");
  }
  const int64_t npix = mwss ? (int64_t)(L + 1) * 2 * L : (int64_t)L * (2 * L - 1);
  if (spin_prints) {
    printf("naxis[0] = %li\n", key_long(h, "NAXIS1", &f));
    printf("naxis[1] = %li\n", key_long(h, "NAXIS2", &f));
  }
  fflush(stdout);
  const long nrows = key_long(h, "NAXIS2", &f);
  if (nrows <= 0 || npix % nrows != 0) fprintf(stderr, "%s: Problem with npix.\n", __FILE__);
  std::vector<std::vector<double>> cols;
  for (int c = 1; c <= ncol; ++c) {
    cols.push_back(read_column(buf, h, c));
    S2G_REQUIRE((int64_t)cols.back().size() >= npix, ERR_INVALID, "the map in the FITS file has fewer samples than L requires");
  }
  for (int c = 0; c < ncol; ++c) memcpy(dst[c], cols[c].data(), sizeof(double) * (size_t)npix);
}

template <class F>
void fits_guard(const char *fn, F &&body) {
  try {
    body();
    set_status(OK, "");
    return;
  } catch (const Error &e) {
    set_status(e.code, std::string(fn) + ": " + e.what());
  } catch (const std::exception &e) {
    set_status(ERR_INVALID, std::string(fn) + ": " + e.what());
  }
  report_failure();
}

}  // namespace
}  // namespace s2g

extern "C" {

int s2let_fits_mw_read_bandlimit(char *filename) {
  long L = -1;
  s2g::fits_guard(__func__, [&] {
    std::vector<char> buf;
    s2g::Hdu h = s2g::open_table(filename, buf);
    bool f;
    L = s2g::key_long(h, "L", &f);
    if (!f) L = -1;  // src/c/s2let_fits.c:41-44
  });
  return (int)L;
}

int s2let_fits_hpx_read_nside(char *filename) {
  long n = -1;
  s2g::fits_guard(__func__, [&] {
    std::vector<char> buf;
    s2g::Hdu h = s2g::open_table(filename, buf);
    bool f;
    n = s2g::key_long(h, "NSIDE", &f);
    if (!f) n = -1;
  });
  return (int)n;
}

void s2let_fits_mw_read_map(double *f, char *file, int L) {
  s2g::fits_guard(__func__, [&] {
    double *d[1] = {f};
    s2g::read_maps(d, 1, file, L, false, false);
  });
}
void s2let_fits_mwss_read_map(double *f, char *file, int L) {
  s2g::fits_guard(__func__, [&] {
    double *d[1] = {f};
    s2g::read_maps(d, 1, file, L, true, false);
  });
}
void s2let_fits_mw_read_spin_maps(double *fQ, double *fU, char *file, int L) {
  s2g::fits_guard(__func__, [&] {
    double *d[2] = {fQ, fU};
    s2g::read_maps(d, 2, file, L, false, true);
  });
}
void s2let_fits_mwss_read_spin_maps(double *fQ, double *fU, char *file, int L) {
  s2g::fits_guard(__func__, [&] {
    double *d[2] = {fQ, fU};
    s2g::read_maps(d, 2, file, L, true, true);
  });
}

void s2let_fits_mw_write_map(char *file, double *f, int L) {
  s2g::fits_guard(__func__, [&] { s2g::write_table(file, L, false, {{"SIGNAL", f}}, (int64_t)L * (2 * L - 1)); });
}
void s2let_fits_mwss_write_map(char *file, double *f, int L) {
  s2g::fits_guard(__func__, [&] { s2g::write_table(file, L, true, {{"SIGNAL", f}}, (int64_t)(L + 1) * 2 * L); });
}
void s2let_fits_mw_write_spin_maps(char *file, double *fQ, double *fU, int L) {
  s2g::fits_guard(__func__, [&] {
    s2g::write_table(file, L, false, {{"Q_POLARISATION", fQ}, {"U_POLARISATION", fU}}, (int64_t)L * (2 * L - 1));
  });
}
void s2let_fits_mwss_write_spin_maps(char *file, double *fQ, double *fU, int L) {
  s2g::fits_guard(__func__, [&] {
    s2g::write_table(file, L, true, {{"Q_POLARISATION", fQ}, {"U_POLARISATION", fU}}, (int64_t)(L + 1) * 2 * L);
  });
}

}  // extern "C"
