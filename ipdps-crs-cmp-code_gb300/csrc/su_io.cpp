// SU ingest and output for the semblance search (host side).
//
// Restates, in this library's own code, what the reference's su_trace / su_cdp /
// su_gather classes do on the path (CRS/OpenMP/src/su_trace.cpp, su_cdp.cpp,
// su_gather.cpp) and its output writer (CRS/OpenMP/src/main.cpp:331-359):
//  * a trace is a 240-byte header followed by ns float32 samples; a short header
//    at end of file ends the input, a short sample block is an error
//    (su_trace.cpp:37-51);
//  * traces whose half-offset exceeds aph are dropped; the test is done on the
//    float half-offsets in the precision of the method's shipped build (float for
//    CMP, double for CRS) (su_gather.cpp:43-47);
//  * traces are grouped by their cdp header, CDPs in ascending cdp order, traces in
//    file order (std::map, su_gather.cpp:38-65); CMP then orders CDPs by
//    decreasing fold with std::sort and the same comparison
//    (CMP/OpenMP/src/su_gather.cpp:68, su_cdp.hpp:53-55), which reproduces the
//    reference's order among equal folds for the same C++ library;
//  * dt is taken from the first trace of the first CDP (su_gather.cpp:103).
// Unlike the reference (whose ns check is an assert compiled out of release
// builds), traces of different ns are rejected.
#include <algorithm>
#include <cerrno>
#include <cstdarg>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "common.h"

namespace semb {

static thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

// Header byte offsets (SEG-Y trace header as declared in su_trace.hpp:42-125).
enum : int {
  kHdrSize = 240,
  kOffCdp = 20,
  kOffOffset = 36,
  kOffScalco = 70,
  kOffSx = 72,
  kOffSy = 76,
  kOffGx = 80,
  kOffGy = 84,
  kOffNs = 114,
  kOffDt = 116,
};

static inline int32_t rd_i32(const unsigned char* h, int off) {
  int32_t v;
  std::memcpy(&v, h + off, 4);
  return v;
}
static inline int16_t rd_i16(const unsigned char* h, int off) {
  int16_t v;
  std::memcpy(&v, h + off, 2);
  return v;
}
static inline uint16_t rd_u16(const unsigned char* h, int off) {
  uint16_t v;
  std::memcpy(&v, h + off, 2);
  return v;
}
static inline void wr_i32(unsigned char* h, int off, int32_t v) { std::memcpy(h + off, &v, 4); }

// su_trace::fscalco (su_trace.cpp:102-107)
static inline float fscalco(int16_t s) {
  if (s == 0) return 1.0f;
  if (s > 0) return (float)s;
  return 1.0f / (float)s;
}

}  // namespace semb

struct semb_survey {
  int32_t method = 0;
  int32_t ns = 0;
  int32_t dt_us = 0;
  std::vector<int64_t> cdp_end;
  std::vector<int32_t> cdp;
  std::vector<int32_t> gx, gy, sx, sy, scalco;
  std::vector<float> samples;
  std::vector<unsigned char> first_hdr;   // [ncdps][240]
};

using namespace semb;

namespace {

struct TraceRef {
  const unsigned char* hdr;
  const unsigned char* data;
};

struct Group {
  int32_t cdp;
  std::vector<TraceRef> traces;
  // su_cdp::operator< : the larger fold sorts first (CMP/OpenMP/include/su_cdp.hpp:53-55)
  bool operator<(const Group& o) const { return traces.size() > o.traces.size(); }
};

int build_survey(const unsigned char* bytes, int64_t nbytes, int32_t method, int32_t aph, semb_survey** out) {
  if (method != SEMB_CMP && method != SEMB_CRS) return fail(SEMB_E_ARG, "unknown method %d", method);
  std::map<int32_t, Group> by_cdp;
  int64_t pos = 0;
  int ns0 = -1;
  const double aph2 = (double)((int64_t)aph * (int64_t)aph);
  while (pos + kHdrSize <= nbytes) {
    const unsigned char* h = bytes + pos;
    const int ns = rd_u16(h, kOffNs);
    const int64_t need = (int64_t)kHdrSize + 4ll * ns;
    if (pos + need > nbytes) return fail(SEMB_E_FORMAT, "Bad input data: trace at byte %lld is truncated", (long long)pos);
    pos += need;
    // half-offset test (su_gather.cpp:44-47): halfoffset_x() = fscalco() * (gx - sx) * 0.5 in float
    const float fs = fscalco(rd_i16(h, kOffScalco));
    const float hxf = (float)(fs * (float)(rd_i32(h, kOffGx) - rd_i32(h, kOffSx)) * 0.5);
    const float hyf = (float)(fs * (float)(rd_i32(h, kOffGy) - rd_i32(h, kOffSy)) * 0.5);
    bool drop;
    if (method == SEMB_CMP) {
      // real = float (CMP/OpenMP/include/utils.hpp:35)
      volatile float a = hxf * hxf;
      volatile float b = hyf * hyf;
      drop = (float)(a + b) > (float)((int32_t)aph * (int32_t)aph);
    } else {
      // real = double (CRS/OpenMP/include/utils.hpp:35)
      const double hx = hxf, hy = hyf;
      volatile double a = hx * hx;
      volatile double b = hy * hy;
      drop = (a + b) > aph2;
    }
    if (drop) continue;
    if (ns0 < 0) ns0 = ns;
    if (ns != ns0) return fail(SEMB_E_FORMAT, "traces with different ns (%d and %d)", ns0, ns);
    const int32_t cdp = rd_i32(h, kOffCdp);
    Group& g = by_cdp[cdp];
    g.cdp = cdp;
    g.traces.push_back(TraceRef{h, h + kHdrSize});
  }
  std::vector<Group> groups;
  groups.reserve(by_cdp.size());
  for (auto& kv : by_cdp) groups.push_back(std::move(kv.second));
  if (method == SEMB_CMP) std::sort(groups.begin(), groups.end());

  semb_survey* s = new (std::nothrow) semb_survey();
  if (!s) return fail(SEMB_E_NOMEM, "out of host memory");
  s->method = method;
  s->ns = ns0 < 0 ? 0 : ns0;
  int64_t ntr = 0;
  for (auto& g : groups) ntr += (int64_t)g.traces.size();
  try {
    s->cdp_end.resize(groups.size());
    s->cdp.resize(groups.size());
    s->gx.resize(ntr);
    s->gy.resize(ntr);
    s->sx.resize(ntr);
    s->sy.resize(ntr);
    s->scalco.resize(ntr);
    s->samples.resize((size_t)ntr * s->ns);
    s->first_hdr.resize(groups.size() * (size_t)kHdrSize);
  } catch (...) {
    delete s;
    return fail(SEMB_E_NOMEM, "out of host memory for %lld traces", (long long)ntr);
  }
  int64_t t = 0;
  for (size_t i = 0; i < groups.size(); ++i) {
    const Group& g = groups[i];
    s->cdp[i] = g.cdp;
    std::memcpy(&s->first_hdr[i * kHdrSize], g.traces[0].hdr, kHdrSize);
    for (const TraceRef& tr : g.traces) {
      s->gx[t] = rd_i32(tr.hdr, kOffGx);
      s->gy[t] = rd_i32(tr.hdr, kOffGy);
      s->sx[t] = rd_i32(tr.hdr, kOffSx);
      s->sy[t] = rd_i32(tr.hdr, kOffSy);
      s->scalco[t] = rd_i16(tr.hdr, kOffScalco);
      std::memcpy(&s->samples[(size_t)t * s->ns], tr.data, 4ull * s->ns);
      ++t;
    }
    s->cdp_end[i] = t;
  }
  s->dt_us = groups.empty() ? 0 : rd_u16(groups[0].traces[0].hdr, kOffDt);
  *out = s;
  return SEMB_OK;
}

}  // namespace

extern "C" {

void semb_params_init(semb_params* p, int32_t method) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->method = method;
  p->mode = SEMB_BATCHED;
  p->storage = SEMB_STORE_F16;
  p->repick = SEMB_REPICK_NEAR_TIES;
  p->repick_gap = 1e-4f;
  p->na = p->nb = 1;
}

int semb_survey_from_bytes(const void* su_bytes, int64_t nbytes, int32_t method, int32_t aph, semb_survey** out) {
  if (!out || (!su_bytes && nbytes > 0) || nbytes < 0) return fail(SEMB_E_ARG, "null argument");
  *out = nullptr;
  return build_survey(static_cast<const unsigned char*>(su_bytes), nbytes, method, aph, out);
}

int semb_survey_load(const char* path, int32_t method, int32_t aph, semb_survey** out) {
  if (!path || !out) return fail(SEMB_E_ARG, "null argument");
  *out = nullptr;
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(SEMB_E_IO, "cannot open %s: %s", path, std::strerror(errno));
  std::vector<unsigned char> bytes;
  unsigned char tmp[1 << 16];
  size_t n;
  try {
    while ((n = std::fread(tmp, 1, sizeof(tmp), f)) > 0) bytes.insert(bytes.end(), tmp, tmp + n);
  } catch (...) {
    std::fclose(f);
    return fail(SEMB_E_NOMEM, "out of host memory reading %s", path);
  }
  const bool err = std::ferror(f) != 0;
  std::fclose(f);
  if (err) return fail(SEMB_E_IO, "read error on %s", path);
  return build_survey(bytes.data(), (int64_t)bytes.size(), method, aph, out);
}

int semb_survey_view(const semb_survey* s, semb_gather_view* v) {
  if (!s || !v) return fail(SEMB_E_ARG, "null argument");
  std::memset(v, 0, sizeof(*v));
  v->ncdps = (int32_t)s->cdp_end.size();
  v->ns = s->ns;
  v->dt_us = s->dt_us;
  v->ntraces = s->cdp_end.empty() ? 0 : s->cdp_end.back();
  v->cdp_end = s->cdp_end.data();
  v->cdp = s->cdp.data();
  v->gx = s->gx.data();
  v->gy = s->gy.data();
  v->sx = s->sx.data();
  v->sy = s->sy.data();
  v->scalco = s->scalco.data();
  v->samples = s->samples.data();
  return SEMB_OK;
}

// Output writer: CMP/OpenMP/src/main.cpp:244-260 and CRS/OpenMP/src/main.cpp:331-359.
// The attribute values use the shipped precision of each method (float for CMP,
// double for CRS) and are stored as float.
int semb_survey_write(const semb_survey* s, const semb_params* p, const int32_t* ctr, const float* str,
                      const float* stk, const char* out_dir) {
  if (!s || !p || !ctr || !str || !stk) return fail(SEMB_E_ARG, "null argument");
  if (p->method != s->method) return fail(SEMB_E_ARG, "method of params and survey differ");
  const std::string dir = (out_dir && *out_dir) ? std::string(out_dir) + "/" : std::string();
  const int ncdps = (int)s->cdp_end.size(), ns = s->ns;
  const char* names_cmp[] = {"cmp.c.su", "cmp.coher.su", "cmp.stack.su"};
  const char* names_crs[] = {"crs.a.su", "crs.b.su", "crs.c.su", "crs.coher.su", "crs.stack.su"};
  const int nout = p->method == SEMB_CMP ? 3 : 5;
  FILE* f[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  for (int k = 0; k < nout; ++k) {
    const std::string path = dir + (p->method == SEMB_CMP ? names_cmp[k] : names_crs[k]);
    f[k] = std::fopen(path.c_str(), "wb");
    if (!f[k]) {
      for (int q = 0; q < k; ++q) std::fclose(f[q]);
      return fail(SEMB_E_IO, "cannot create %s: %s", path.c_str(), std::strerror(errno));
    }
  }
  // attribute grids exactly as the writer computes them
  std::vector<float> vals((size_t)ns);
  unsigned char hdr0[kHdrSize], hdr[kHdrSize];
  bool ok = true;
  for (int i = 0; i < ncdps && ok; ++i) {
    // attribute files (c, or a/b/c): the first trace's header with offset 0 and
    // source and receiver at the integer midpoint; coherence and stack files: the
    // first trace's header unchanged (CMP/OpenMP/src/main.cpp:245-251,
    // CRS/OpenMP/src/main.cpp:332-346)
    std::memcpy(hdr0, &s->first_hdr[(size_t)i * kHdrSize], kHdrSize);
    std::memcpy(hdr, hdr0, kHdrSize);
    const int32_t sx0 = rd_i32(hdr, kOffSx), gx0 = rd_i32(hdr, kOffGx);
    const int32_t sy0 = rd_i32(hdr, kOffSy), gy0 = rd_i32(hdr, kOffGy);
    wr_i32(hdr, kOffOffset, 0);
    const int32_t mx = (int32_t)(((int64_t)sx0 + gx0) >> 1);
    const int32_t my = (int32_t)(((int64_t)sy0 + gy0) >> 1);
    wr_i32(hdr, kOffSx, mx);
    wr_i32(hdr, kOffGx, mx);
    wr_i32(hdr, kOffSy, my);
    wr_i32(hdr, kOffGy, my);
    const int32_t* c = ctr + (size_t)i * ns;
    for (int k = 0; k < nout && ok; ++k) {
      const float* data = nullptr;
      if (p->method == SEMB_CMP) {
        if (k == 0) {
          const float c0 = (float)(p->c0 * kFactor), c1 = (float)(p->c1 * kFactor);
          volatile float diff = c1 - c0;
          const float inc = diff * (1.0f / (float)p->nc);
          for (int q = 0; q < ns; ++q) {
            volatile float prod = inc * (float)c[q];
            vals[q] = c[q] < 0 ? 0.0f : (float)((double)(float)(c0 + prod) / kFactor);
          }
          data = vals.data();
        } else {
          data = (k == 1 ? str : stk) + (size_t)i * ns;
        }
      } else {
        const int na = p->na, nb = p->nb, nc = p->nc;
        if (k < 3) {
          const double a0 = p->a0, b0 = p->b0, c0 = p->c0 * kFactor;
          const double inc_a = (p->a1 - a0) * (1.0 / (double)na);
          const double inc_b = (p->b1 - b0) * (1.0 / (double)nb);
          const double inc_c = (p->c1 * kFactor - c0) * (1.0 / (double)nc);
          for (int q = 0; q < ns; ++q) {
            volatile double prod;
            if (k == 0) {
              prod = inc_a * (double)(c[q] / (nc * nb));
              vals[q] = (float)(a0 + prod);
            } else if (k == 1) {
              prod = inc_b * (double)((c[q] / nc) % nb);
              vals[q] = (float)(b0 + prod);
            } else {
              prod = inc_c * (double)(c[q] % nc);
              vals[q] = (float)((c0 + prod) / kFactor);
            }
          }
          data = vals.data();
        } else {
          data = (k == 3 ? str : stk) + (size_t)i * ns;
        }
      }
      const bool attribute = k < nout - 2;
      ok = std::fwrite(attribute ? hdr : hdr0, 1, kHdrSize, f[k]) == (size_t)kHdrSize &&
           std::fwrite(data, sizeof(float), (size_t)ns, f[k]) == (size_t)ns;
    }
  }
  for (int k = 0; k < nout; ++k) ok = (std::fclose(f[k]) == 0) && ok;
  return ok ? SEMB_OK : fail(SEMB_E_IO, "write error");
}

int semb_survey_write_abc(const semb_survey* s, const float* a, const float* b, const float* c, const float* str,
                          const float* stk, const char* out_dir) {
  if (!s || !a || !b || !c || !str || !stk) return fail(SEMB_E_ARG, "null argument");
  if (s->method != SEMB_CRS) return fail(SEMB_E_ARG, "explicit A, B, C outputs are CRS files");
  const std::string dir = (out_dir && *out_dir) ? std::string(out_dir) + "/" : std::string();
  const char* names[] = {"crs.a.su", "crs.b.su", "crs.c.su", "crs.coher.su", "crs.stack.su"};
  const float* data[] = {a, b, c, str, stk};
  FILE* f[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  for (int k = 0; k < 5; ++k) {
    const std::string path = dir + names[k];
    f[k] = std::fopen(path.c_str(), "wb");
    if (!f[k]) {
      for (int q = 0; q < k; ++q) std::fclose(f[q]);
      return fail(SEMB_E_IO, "cannot create %s: %s", path.c_str(), std::strerror(errno));
    }
  }
  const int ncdps = (int)s->cdp_end.size(), ns = s->ns;
  unsigned char hdr0[kHdrSize], hdr[kHdrSize];
  bool ok = true;
  for (int i = 0; i < ncdps && ok; ++i) {
    // headers as semb_survey_write: parameter files with offset 0 and the integer
    // midpoint, coherence and stack files with the first trace's header
    std::memcpy(hdr0, &s->first_hdr[(size_t)i * kHdrSize], kHdrSize);
    std::memcpy(hdr, hdr0, kHdrSize);
    const int32_t mx = (int32_t)(((int64_t)rd_i32(hdr, kOffSx) + rd_i32(hdr, kOffGx)) >> 1);
    const int32_t my = (int32_t)(((int64_t)rd_i32(hdr, kOffSy) + rd_i32(hdr, kOffGy)) >> 1);
    wr_i32(hdr, kOffOffset, 0);
    wr_i32(hdr, kOffSx, mx);
    wr_i32(hdr, kOffGx, mx);
    wr_i32(hdr, kOffSy, my);
    wr_i32(hdr, kOffGy, my);
    for (int k = 0; k < 5 && ok; ++k)
      ok = std::fwrite(k < 3 ? hdr : hdr0, 1, kHdrSize, f[k]) == (size_t)kHdrSize &&
           std::fwrite(data[k] + (size_t)i * ns, sizeof(float), (size_t)ns, f[k]) == (size_t)ns;
  }
  for (int k = 0; k < 5; ++k) ok = (std::fclose(f[k]) == 0) && ok;
  return ok ? SEMB_OK : fail(SEMB_E_IO, "write error");
}

int semb_survey_write_attr(const semb_survey* s, const char* name, const float* data, const char* out_dir) {
  if (!s || !name || !*name || !data) return fail(SEMB_E_ARG, "null argument");
  const std::string dir = (out_dir && *out_dir) ? std::string(out_dir) + "/" : std::string();
  const std::string path = dir + name;
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return fail(SEMB_E_IO, "cannot create %s: %s", path.c_str(), std::strerror(errno));
  const int ncdps = (int)s->cdp_end.size(), ns = s->ns;
  bool ok = true;
  for (int i = 0; i < ncdps && ok; ++i)
    ok = std::fwrite(&s->first_hdr[(size_t)i * kHdrSize], 1, kHdrSize, f) == (size_t)kHdrSize &&
         std::fwrite(data + (size_t)i * ns, sizeof(float), (size_t)ns, f) == (size_t)ns;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? SEMB_OK : fail(SEMB_E_IO, "write error");
}

void semb_survey_free(semb_survey* s) { delete s; }

const char* semb_strerror(int code) {
  switch (code) {
    case SEMB_OK: return "ok";
    case SEMB_E_ARG: return "invalid argument";
    case SEMB_E_IO: return "i/o error";
    case SEMB_E_FORMAT: return "malformed SU data";
    case SEMB_E_WINDOW: return "semblance window too large";
    case SEMB_E_NOMEM: return "out of memory";
    case SEMB_E_CUDA: return "CUDA error";
    case SEMB_E_TIMEOUT: return "device wait timed out";
    case SEMB_E_STATE: return "call out of order";
    case SEMB_E_NODEV: return "no usable CUDA device";
    case SEMB_E_BOUNDS: return "bounds check failed (checked build)";
    default: return "unknown error";
  }
}

const char* semb_last_error(void) { return semb::g_last_error.c_str(); }

int32_t semb_abi_version(void) { return SEMB_ABI_VERSION; }

}  // extern "C"
