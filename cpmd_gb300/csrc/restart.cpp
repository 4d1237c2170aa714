// RESTART wavefunction file of the Gamma point: host-side writer and reader
// of the reference's restart format (wv30_utils.mod.F90, rv30_utils.mod.F90,
// wfnio_utils.mod.F90, wr30wfn_utils.mod.F90, compress.F90).
//
// Layout.  A Fortran unformatted sequential file: every WRITE statement is one
// record framed by its byte length as a 4-byte integer before and after the
// data (the STREAM variant has no frames; its section headers carry the byte
// position of the section end instead).  Section 1 is one 80-character record
// (" STUTTGART VERSION 3.0").  Sections 2..99 each start with a record
// (irecord int32, fpos int64) and are followed by irecord records (0: section
// empty; the count is what lets a reader skip a section it does not parse);
// section 9, the states, uses a negative count -(2 n + 3) for the
// w_wfnio format: (iwfntype), (n, ngwks, icompr, scale), (tlsd, nsup, nsdown),
// then per state (nx) and the 2 nx 32-bit words of the compressed coefficients
// in the global G order.
//
// Compression (compress.F90, the spack/sunpack variant built on Linux):
// icompr 1 stores the FP64 values as is (nx = number of doubles); icompr =
// 2, 4, 8 stores nb = 64/icompr bit fixed-point values v = NINT(x fx) offset by
// 2^(nb-1), fx = (2^(nb-1) - 1) / scale, packed into 32-bit words high part
// first, and the reader decodes (nx - 1) icompr values (so the last word pair of
// a compressed state is not read back, as in the reference).  scale is the
// modulus of the coefficient with the largest |Re| + |Im| over all states
// (izamax, wfnio_utils.mod.F90:130-135).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cpmd_gb300.h"

namespace {

constexpr int kHeaderLen = 80;
const char kHeader[] = " STUTTGART VERSION 3.0";

// ---------------------------------------------------------------- writing
struct RecWriter {
  FILE* f = nullptr;
  bool ok = true;
  explicit RecWriter(const char* path) : f(std::fopen(path, "wb")) { ok = f != nullptr; }
  ~RecWriter() {
    if (f) std::fclose(f);
  }
  // one record from consecutive pieces
  void rec(std::initializer_list<std::pair<const void*, size_t>> parts) {
    size_t n = 0;
    for (const auto& p : parts) n += p.second;
    if (!ok || n > 0x7FFFFFFFull) {
      ok = false;
      return;
    }
    const int32_t m = (int32_t)n;
    ok = std::fwrite(&m, 4, 1, f) == 1;
    for (const auto& p : parts)
      if (ok && p.second) ok = std::fwrite(p.first, 1, p.second, f) == p.second;
    if (ok) ok = std::fwrite(&m, 4, 1, f) == 1;
  }
  void section(int32_t irecord) {
    const int64_t fpos = 0;
    rec({{&irecord, 4}, {&fpos, 8}});
  }
  bool close() {
    if (f && std::fclose(f) != 0) ok = false;
    f = nullptr;
    return ok;
  }
};

// NINT: nearest integer, halves away from zero
inline long long nint(double x) { return std::llround(x); }

// compress.F90 (icompr 1 or 2) of one state's 2 ngw doubles into 32-bit words;
// returns nx (the count written as the state's first record)
int32_t compress_state(const double* a, int64_t n, int icompr, double scale, std::vector<uint32_t>& words) {
  if (icompr == 1) {
    words.resize((size_t)(2 * n));
    std::memcpy(words.data(), a, (size_t)n * 8);
    return (int32_t)n;
  }
  // nb = 32: m = n + mod(n, 2) values, nx = m / 2, one value per word
  const int64_t m = n + n % 2;
  const double fx = scale > 0.0 ? 2147483647.0 / scale : 0.0;
  words.assign((size_t)m, 0u);
  for (int64_t i = 0; i < n; ++i) {
    long long v = nint(a[i] * fx);
    if (v > 2147483647ll) v = 2147483647ll;  // |x| > scale is possible with the izamax scale
    if (v < -2147483647ll) v = -2147483647ll;
    words[(size_t)i] = (uint32_t)(v + 2147483648ll);
  }
  for (int64_t i = n; i < m; ++i) words[(size_t)i] = 2147483648u;
  return (int32_t)(m / 2);
}

// the modulus of the element with the largest |Re| + |Im| (first on ties)
double izamax_scale(const double* c0, int ldc, int ngw, int nstate) {
  double best = -1.0, re = 0.0, im = 0.0;
  for (int s = 0; s < nstate; ++s)
    for (int g = 0; g < ngw; ++g) {
      const double* z = c0 + 2 * ((size_t)s * ldc + g);
      const double a = std::fabs(z[0]) + std::fabs(z[1]);
      if (a > best) {
        best = a;
        re = z[0];
        im = z[1];
      }
    }
  return std::hypot(re, im);
}

// the largest |component| of the real view (idamax, wr30wfn_utils.mod.F90:636-637)
double idamax_scale(const double* c, int ldc, int ngw, int nstate) {
  double best = 0.0;
  for (int s = 0; s < nstate; ++s)
    for (int i = 0; i < 2 * ngw; ++i) best = std::max(best, std::fabs(c[2 * (size_t)s * ldc + i]));
  return best;
}

int write_restart(const char* path, const gbcp_restart* r) {
  if (!path || !r || r->nsp < 0 || r->nat < 0 || r->nstate < 0) return GBCP_ERR_ARG;
  if ((r->nsp > 0 && !r->na) || (r->nat > 0 && !r->tau0)) return GBCP_ERR_ARG;
  const bool states = r->nstate > 0 && r->c0;
  if (states && (r->ngw < 1 || r->ldc < r->ngw)) return GBCP_ERR_ARG;
  if (states && r->icompr != 1 && r->icompr != 2) return GBCP_ERR_ARG;
  const int32_t ngwks = r->ngwks > 0 ? r->ngwks : r->ngw;
  if (states && ngwks != r->ngw) return GBCP_ERR_ARG;
  RecWriter w(path);
  if (!w.ok) return GBCP_ERR_IO;
  // section 1
  char hdr[kHeaderLen];
  std::memset(hdr, ' ', sizeof hdr);
  std::memcpy(hdr, kHeader, sizeof kHeader - 1);
  w.rec({{hdr, sizeof hdr}});
  // section 2: symmetry and cell
  w.section(2);
  w.rec({{&r->ibrav, 4}, {&r->indpg, 4}});
  w.rec({{r->celldm, 48}});
  // section 3: species
  w.section(2);
  w.rec({{&r->nsp, 4}});
  w.rec({{r->na, 4 * (size_t)r->nsp}});
  // sections 4, 5, 6: coordinates, velocities, initial coordinates
  for (const double* t : {(const double*)r->tau0, (const double*)r->taum, (const double*)r->taui}) {
    if (t && r->nat > 0) {
      w.section(r->nat);
      for (int ia = 0; ia < r->nat; ++ia) w.rec({{t + 3 * (size_t)ia, 24}});
    } else {
      w.section(0);
    }
  }
  // section 7: cutoff, dual, electrons, mesh
  w.section(1);
  const int32_t dual = r->dual ? 1 : 0;
  w.rec({{&r->ecut, 8}, {&r->cdual, 8}, {&dual, 4}, {&r->nel, 4}, {&r->nr1s, 4}, {&r->nr2s, 4}, {&r->nr3s, 4}});
  // section 8: states, k points (0 = Gamma), plane-wave counts
  w.section(1);
  const int32_t nkpts0 = 0;
  w.rec({{&r->nstate, 4}, {&nkpts0, 4}, {&ngwks, 4}, {&r->ngwls, 4}, {&r->nhgs, 4}, {&r->nhgls, 4}});
  // section 9: the states (w_wfnio, type 1)
  if (states) {
    const int32_t irecord = -(2 * r->nstate + 3);
    const int64_t pos = -1;
    w.rec({{&irecord, 4}, {&pos, 8}});
    const int32_t iwfntype = 1, icompr = r->icompr, tlsd = 0, nsup = 0, nsdown = 0;
    const double scale = izamax_scale(r->c0, r->ldc, r->ngw, r->nstate);
    w.rec({{&iwfntype, 4}});
    w.rec({{&r->nstate, 4}, {&ngwks, 4}, {&icompr, 4}, {&scale, 8}});
    w.rec({{&tlsd, 4}, {&nsup, 4}, {&nsdown, 4}});
    std::vector<uint32_t> words;
    for (int s = 0; s < r->nstate && w.ok; ++s) {
      const int32_t nx = compress_state(r->c0 + 2 * (size_t)s * r->ldc, 2 * (int64_t)ngwks, icompr, scale, words);
      w.rec({{&nx, 4}});
      w.rec({{words.data(), 8 * (size_t)nx}});
    }
  } else {
    w.section(0);
  }
  // section 10: wavefunction velocities (wr30wfn 'NIL')
  if (r->cm && states) {
    const int32_t icompr = r->icompr;
    const double scale = idamax_scale(r->cm, r->ldc, r->ngw, r->nstate);
    w.section(2 * r->nstate + 1);
    w.rec({{&r->nstate, 4}, {&ngwks, 4}, {&icompr, 4}, {&scale, 8}});
    std::vector<uint32_t> words;
    for (int s = 0; s < r->nstate && w.ok; ++s) {
      const int32_t nx = compress_state(r->cm + 2 * (size_t)s * r->ldc, 2 * (int64_t)ngwks, icompr, scale, words);
      w.rec({{&nx, 4}});
      w.rec({{words.data(), 8 * (size_t)nx}});
    }
  } else {
    w.section(0);
  }
  // sections 11 .. 22: empty
  for (int sec = 11; sec <= 22; ++sec) w.section(0);
  // section 23: occupation numbers (one k point)
  if (r->f && r->nstate > 0) {
    w.section(1);
    w.rec({{r->f, 8 * (size_t)r->nstate}});
  } else {
    w.section(0);
  }
  // section 24: Fermi energy, eigenvalues
  if (r->eigv && r->nstate > 0) {
    w.section(2);
    w.rec({{&r->amu, 8}});
    w.rec({{r->eigv, 8 * (size_t)r->nstate}});
  } else {
    w.section(0);
  }
  // sections 25 .. 99: empty
  for (int sec = 25; sec <= 99; ++sec) w.section(0);
  return w.close() ? GBCP_OK : GBCP_ERR_IO;
}

// ---------------------------------------------------------------- reading
struct RecReader {
  FILE* f = nullptr;
  bool stream = false;  // STREAM file: no record frames
  bool ok = true;
  int64_t size = 0;      // file length: no record or state may claim more than what is left
  explicit RecReader(const char* path) : f(std::fopen(path, "rb")) {
    ok = f != nullptr;
    if (ok && std::fseek(f, 0, SEEK_END) == 0) {
      size = (int64_t)std::ftell(f);
      ok = size >= 0 && std::fseek(f, 0, SEEK_SET) == 0;
    } else {
      ok = false;
    }
  }
  int64_t left() const { return f ? size - (int64_t)std::ftell(f) : 0; }
  ~RecReader() {
    if (f) std::fclose(f);
  }
  bool raw(void* dst, size_t n) {
    if (ok && n) ok = std::fread(dst, 1, n, f) == n;
    return ok;
  }
  // the next record; in a STREAM file the caller names its size (`want`)
  bool next(std::vector<uint8_t>& buf, size_t want) {
    if (!ok) return false;
    if (stream) {
      if ((int64_t)want > left()) return ok = false;
      buf.resize(want);
      return raw(buf.data(), want);
    }
    int32_t m = 0, t = 0;
    if (!raw(&m, 4) || m < 0) return ok = false;  // negative: a split record, not written by the reference here
    if ((int64_t)m + 4 > left()) return ok = false;  // longer than the rest of the file: corrupt
    buf.resize((size_t)m);
    if (!raw(buf.data(), (size_t)m) || !raw(&t, 4) || t != m) return ok = false;
    return true;
  }
  // a record of at least `want` bytes whose first `want` bytes go to dst
  bool read(void* dst, size_t want, std::vector<uint8_t>& buf) {
    if (!next(buf, want) || buf.size() < want) return ok = false;
    std::memcpy(dst, buf.data(), want);
    return true;
  }
  // section header: (irecord) [+ fpos, the STREAM end position, 1-based]
  bool section(int32_t& irecord, int64_t& fpos, std::vector<uint8_t>& buf) {
    fpos = 0;
    if (!next(buf, 12) || buf.size() < 4) return ok = false;
    std::memcpy(&irecord, buf.data(), 4);
    if (buf.size() >= 12) std::memcpy(&fpos, buf.data() + 4, 8);
    return true;
  }
  // skip a section whose records are not read (fskip of rv30, or the seek of a STREAM file)
  bool skip(int32_t irecord, int64_t fpos, std::vector<uint8_t>& buf) {
    if (stream) return ok = ok && fpos > 0 && std::fseek(f, (long)(fpos - 1), SEEK_SET) == 0;
    for (int32_t i = 0; i < (irecord < 0 ? -irecord : irecord) && ok; ++i) next(buf, 0);
    return ok;
  }
};

// decompr + sunpack of one state's words into a (capacity na doubles); returns
// the number of values decoded, or -1 if the record does not fit
int64_t decompress_state(const uint32_t* w, int32_t nx, int icompr, double scale, double* a, int64_t na) {
  if (icompr == 1) {
    if ((int64_t)nx > na) return -1;
    std::memcpy(a, w, (size_t)nx * 8);
    return nx;
  }
  const int nb = 64 / icompr;
  const int64_t n = ((int64_t)nx - 1) * icompr;
  if (n > na || n < 0) return -1;
  const double fx = scale / (std::ldexp(1.0, nb - 1) - 1.0);
  for (int64_t i = 0; i < n; ++i) {
    int64_t u;
    if (nb == 32) {
      u = (int64_t)(int32_t)(w[i] ^ 0x80000000u);  // the value minus the offset 2^31, modulo 2^32
    } else if (nb == 16) {
      const uint32_t x = w[i / 2];
      u = (int64_t)((i % 2 == 0) ? (x >> 16) : (x & 0xFFFFu)) - 32768;
    } else {
      const uint32_t x = w[i / 4];
      u = (int64_t)((x >> (24 - 8 * (i % 4))) & 0xFFu) - 128;
    }
    a[i] = (double)u * fx;
  }
  return n;
}

// The per-state records (nx), (2 nx words) of n0 states: the first min(n0, cap)
// decoded into dst (ngw rows of leading dimension ld; rows beyond the file's
// ngwks0 zeroed, as rdwfn does), the rest skipped (STREAM: to the section end).
int read_states(RecReader& rd, std::vector<uint8_t>& buf, int n0, int ngwks0, int icompr, double scale,
                double* dst, int ld, int ngw, int cap, int64_t fpos, int32_t* nread) {
  const int nr = dst ? (n0 < cap ? n0 : cap) : 0;
  // a state of ngwks0 coefficients takes at least 2 ngwks0 bytes (icompr 8), so a
  // count beyond what is left of the file is corrupt (and must not size a buffer)
  if (nr > 0 && 2 * (int64_t)ngwks0 > rd.left()) return GBCP_ERR_IO;
  std::vector<double> ca(nr > 0 ? 2 * (size_t)ngwks0 + 16 : 0);
  *nread = 0;
  for (int s = 0; s < nr; ++s) {
    int32_t nx = 0;
    if (!rd.read(&nx, 4, buf) || nx < 0) return GBCP_ERR_IO;
    if (!rd.next(buf, 8 * (size_t)nx) || buf.size() < 8 * (size_t)nx) return GBCP_ERR_IO;
    std::fill(ca.begin(), ca.end(), 0.0);
    if (decompress_state(reinterpret_cast<const uint32_t*>(buf.data()), nx, icompr, scale, ca.data(),
                         2 * (int64_t)ngwks0) < 0)
      return GBCP_ERR_IO;
    double* c = dst + 2 * (size_t)s * ld;
    const int m = ngwks0 < ngw ? ngwks0 : ngw;
    for (int64_t i = 0; i < 2 * (int64_t)m; ++i) {
      if (!std::isfinite(ca[(size_t)i])) return GBCP_ERR_NONFINITE;  // rdwfn stops on non-finite values
      c[i] = ca[(size_t)i];
    }
    for (int64_t i = 2 * (int64_t)m; i < 2 * (int64_t)ngw; ++i) c[i] = 0.0;
    *nread = s + 1;
  }
  if (rd.stream) {
    if (nr < n0 && !rd.skip(0, fpos, buf)) return GBCP_ERR_IO;
  } else {
    for (int s = nr; s < n0; ++s)
      if (!rd.next(buf, 0) || !rd.next(buf, 0)) return GBCP_ERR_IO;
  }
  return GBCP_OK;
}

// w_wfnio type-1 records after a negative section count: (iwfntype),
// (n, ngwks, icompr, scale), (tlsd, nsup, nsdown), then the states
int read_wfnio(RecReader& rd, std::vector<uint8_t>& buf, double* dst, int ld, int ngw, int cap, int64_t fpos,
               int32_t* n0_out, int32_t* icompr_out, double* scale_out, int32_t* nread) {
  int32_t iwfntype = 0;
  if (!rd.read(&iwfntype, 4, buf)) return GBCP_ERR_IO;
  if (iwfntype != 1) return GBCP_ERR_UNSUPPORTED;  // 9: broken-symmetry pair of wavefunctions
  if (!rd.next(buf, 20) || buf.size() < 20) return GBCP_ERR_IO;
  int32_t n0, ngwks0, icompr;
  double scale;
  std::memcpy(&n0, buf.data(), 4);
  std::memcpy(&ngwks0, buf.data() + 4, 4);
  std::memcpy(&icompr, buf.data() + 8, 4);
  std::memcpy(&scale, buf.data() + 12, 8);
  if (n0 < 0 || ngwks0 < 0 || (icompr != 1 && icompr != 2 && icompr != 4 && icompr != 8)) return GBCP_ERR_IO;
  if (!rd.next(buf, 12) || buf.size() < 12) return GBCP_ERR_IO;  // tlsd, nsup, nsdown
  *n0_out = n0;
  *icompr_out = icompr;
  *scale_out = scale;
  return read_states(rd, buf, n0, ngwks0, icompr, scale, dst, ld, ngw, cap, fpos, nread);
}

int read_restart(const char* path, gbcp_restart* r) {
  if (!path || !r) return GBCP_ERR_ARG;
  if (r->c0 && (r->ngw < 1 || r->ldc < r->ngw || r->nstate_cap < 0)) return GBCP_ERR_ARG;
  RecReader rd(path);
  if (!rd.ok) return GBCP_ERR_IO;
  std::vector<uint8_t> buf;
  r->sections = 0;
  r->nstate_read = 0;
  r->nstate_file = 0;
  // section 1: framed 80-byte header, or the raw header of a STREAM file
  int32_t first = 0;
  if (!rd.raw(&first, 4)) return GBCP_ERR_IO;
  if (first == kHeaderLen) {
    char h[kHeaderLen];
    int32_t t = 0;
    if (!rd.raw(h, kHeaderLen) || !rd.raw(&t, 4) || t != kHeaderLen) return GBCP_ERR_IO;
    if (std::string(h, kHeaderLen).find("STUTTGART") == std::string::npos) return GBCP_ERR_IO;
  } else {
    char h[kHeaderLen];
    std::memcpy(h, &first, 4);
    if (!rd.raw(h + 4, kHeaderLen - 4)) return GBCP_ERR_IO;
    const std::string s(h, kHeaderLen);
    if (s.find("STUTTGART") == std::string::npos || s.find("STREAM") == std::string::npos) return GBCP_ERR_IO;
    rd.stream = true;
  }
  r->sections |= 1;
  int32_t irecord = 0;
  int64_t fpos = 0;
  // section 2: ibrav, indpg; celldm
  if (!rd.section(irecord, fpos, buf)) return GBCP_ERR_IO;
  if (irecord == 2) {
    int32_t v[2];
    if (!rd.read(v, 8, buf) || !rd.read(r->celldm, 48, buf)) return GBCP_ERR_IO;
    r->ibrav = v[0];
    r->indpg = v[1];
    r->sections |= 1 << 1;
  } else if (!rd.skip(irecord, fpos, buf)) {
    return GBCP_ERR_IO;
  }
  // section 3: nsp; na(1:nsp)
  if (!rd.section(irecord, fpos, buf)) return GBCP_ERR_IO;
  r->nat = 0;
  r->nsp = 0;
  if (irecord == 2) {
    if (!rd.read(&r->nsp, 4, buf) || r->nsp < 0) return GBCP_ERR_IO;
    if (!rd.next(buf, 4 * (size_t)r->nsp) || buf.size() < 4 * (size_t)r->nsp) return GBCP_ERR_IO;
    for (int i = 0; i < r->nsp; ++i) {
      int32_t n;
      std::memcpy(&n, buf.data() + 4 * i, 4);
      if (n < 0) return GBCP_ERR_IO;
      r->nat += n;
      if (r->na) r->na[i] = n;
    }
    r->sections |= 1 << 2;
  } else if (!rd.skip(irecord, fpos, buf)) {
    return GBCP_ERR_IO;
  }
  // sections 4, 5, 6: nat records of (x, y, z)
  double* dst[3] = {r->tau0, r->taum, r->taui};
  for (int k = 0; k < 3; ++k) {
    if (!rd.section(irecord, fpos, buf)) return GBCP_ERR_IO;
    if (irecord > 0 && irecord == r->nat) {
      for (int ia = 0; ia < r->nat; ++ia) {
        double x[3];
        if (!rd.read(x, 24, buf)) return GBCP_ERR_IO;
        if (dst[k]) std::memcpy(dst[k] + 3 * (size_t)ia, x, 24);
      }
      r->sections |= 1 << (3 + k);
    } else if (!rd.skip(irecord, fpos, buf)) {
      return GBCP_ERR_IO;
    }
  }
  // section 7: ecut, cdual, dual, nel, nr1s, nr2s, nr3s
  if (!rd.section(irecord, fpos, buf)) return GBCP_ERR_IO;
  if (irecord == 1) {
    if (!rd.next(buf, 36) || buf.size() < 36) return GBCP_ERR_IO;
    std::memcpy(&r->ecut, buf.data(), 8);
    std::memcpy(&r->cdual, buf.data() + 8, 8);
    int32_t v[5];
    std::memcpy(v, buf.data() + 16, 20);
    r->dual = v[0] != 0;
    r->nel = v[1];
    r->nr1s = v[2];
    r->nr2s = v[3];
    r->nr3s = v[4];
    r->sections |= 1 << 6;
  } else if (!rd.skip(irecord, fpos, buf)) {
    return GBCP_ERR_IO;
  }
  // section 8: n, nkpts, ngwks, ngwls, nhgs, nhgls
  if (!rd.section(irecord, fpos, buf)) return GBCP_ERR_IO;
  if (irecord == 1) {
    int32_t v[6];
    if (!rd.read(v, 24, buf)) return GBCP_ERR_IO;
    r->nstate = v[0];
    r->nkpts = v[1];
    r->ngwks = v[2];
    r->ngwls = v[3];
    r->nhgs = v[4];
    r->nhgls = v[5];
    r->sections |= 1 << 7;
    if (r->nkpts != 0) return GBCP_ERR_UNSUPPORTED;  // k points: not the Gamma-point path
  } else if (!rd.skip(irecord, fpos, buf)) {
    return GBCP_ERR_IO;
  }
  // section 9: the states
  if (!rd.section(irecord, fpos, buf)) return GBCP_ERR_IO;
  if (irecord > 0) return GBCP_ERR_UNSUPPORTED;  // the older wr30wfn layout
  if (irecord < 0) {
    const int rc = read_wfnio(rd, buf, r->c0, r->ldc, r->ngw, r->nstate_cap, fpos, &r->nstate_file, &r->icompr,
                              &r->scale, &r->nstate_read);
    if (rc) return rc;
    r->sections |= 1 << 8;
  }
  // section 10 (velocities), 11 .. 22 skipped by their record counts, 23, 24; the file may end after 9
  r->ncm_read = 0;
  for (int sec = 10; sec <= 24; ++sec) {
    if (std::feof(rd.f) || std::fgetc(rd.f) == EOF) break;
    std::fseek(rd.f, -1, SEEK_CUR);
    if (!rd.section(irecord, fpos, buf)) return GBCP_ERR_IO;
    if (sec == 10 && irecord > 0) {  // wr30wfn: (n, ngwks, icompr, scale), then the states
      if (!rd.next(buf, 20) || buf.size() < 20) return GBCP_ERR_IO;
      int32_t n0, ngwks0, icompr;
      double scale;
      std::memcpy(&n0, buf.data(), 4);
      std::memcpy(&ngwks0, buf.data() + 4, 4);
      std::memcpy(&icompr, buf.data() + 8, 4);
      std::memcpy(&scale, buf.data() + 12, 8);
      if (n0 < 0 || ngwks0 < 0 || irecord != 2 * n0 + 1 || (icompr != 1 && icompr != 2 && icompr != 4 && icompr != 8))
        return GBCP_ERR_IO;
      const int rc = read_states(rd, buf, n0, ngwks0, icompr, scale, r->cm, r->ldc, r->ngw, r->nstate_cap, fpos,
                                 &r->ncm_read);
      if (rc) return rc;
      r->sections |= 1 << 9;
    } else if (sec == 10 && irecord < 0) {  // the w_wfnio layout
      int32_t n0, icompr;
      double scale;
      const int rc = read_wfnio(rd, buf, r->cm, r->ldc, r->ngw, r->nstate_cap, fpos, &n0, &icompr, &scale,
                                &r->ncm_read);
      if (rc) return rc;
      r->sections |= 1 << 9;
    } else if (sec == 23 && irecord >= 1 && r->nstate > 0) {  // occupations of the first k point
      if (!rd.next(buf, 8 * (size_t)r->nstate) || buf.size() < 8 * (size_t)r->nstate) return GBCP_ERR_IO;
      if (r->f) std::memcpy(r->f, buf.data(), 8 * (size_t)r->nstate);
      r->sections |= 1 << 22;
      if (!rd.stream && irecord > 1 && !rd.skip(irecord - 1, 0, buf)) return GBCP_ERR_IO;
      if (rd.stream && irecord > 1 && !rd.skip(irecord, fpos, buf)) return GBCP_ERR_IO;
    } else if (sec == 24 && irecord >= 2 && r->nstate > 0) {  // amu, then eigenvalues of the first k point
      if (!rd.read(&r->amu, 8, buf)) return GBCP_ERR_IO;
      if (!rd.next(buf, 8 * (size_t)r->nstate) || buf.size() < 8 * (size_t)r->nstate) return GBCP_ERR_IO;
      if (r->eigv) std::memcpy(r->eigv, buf.data(), 8 * (size_t)r->nstate);
      r->sections |= 1 << 23;
      if (!rd.stream && irecord > 2 && !rd.skip(irecord - 2, 0, buf)) return GBCP_ERR_IO;
      if (rd.stream && irecord > 2 && !rd.skip(irecord, fpos, buf)) return GBCP_ERR_IO;
    } else if (irecord != 0 && !rd.skip(irecord, fpos, buf)) {
      return GBCP_ERR_IO;
    }
  }
  return GBCP_OK;
}

}  // namespace

// No C++ exception may cross the C ABI into a Fortran or C caller: a failed
// allocation (or any other exception) becomes GBCP_ERR_IO.
extern "C" int gbcp_restart_write(const char* path, const gbcp_restart* r) {
  try {
    return write_restart(path, r);
  } catch (...) {
    return GBCP_ERR_IO;
  }
}
extern "C" int gbcp_restart_read(const char* path, gbcp_restart* r) {
  try {
    return read_restart(path, r);
  } catch (...) {
    return GBCP_ERR_IO;
  }
}
