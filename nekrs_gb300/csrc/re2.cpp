// Mesh ingestion: Nek5000 binary .re2 files and the vertex numbering that
// parCon (parRSB) derives from their coordinates.  Host code only.
//
// File layout (Nek5000 core/reader_re2.f: read_re2_hdr :543-620,
// readp_re2_mesh :68-157, readp_re2_curve :159-286, readp_re2_bc :288-428,
// buf_to_xyz / buf_to_curve / buf_to_bc :430-541; nekRS
// src/io/re2Reader.cpp:4-41 for the header check):
//   80-byte ASCII header  "#v002" i9 nelgt, i3 ndim, i9 nelgv (v004: free
//                         format, then the number of boundary sections)
//   4-byte float          6.54321, the byte-order test
//   nelgt element records group, x[8], y[8], z[8]  (8-byte words for v002+,
//                         pre-processor corner order: counter-clockwise bottom
//                         face, then top face)
//   curve section         count, then records (element, face, p[5], type)
//   boundary sections     per field: count, then records (element, face,
//                         p[5], 3-character code in one 8-byte word), in
//                         element order; faces without a record are 'E  '.
// Element and face numbers are stored as floating-point words, 1-based.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "nekrs_gb300.h"
#include "nrsg_internal.hpp"

using nrsg::Error;

namespace {

// hypercube corner v = i + 2j + 4k  <-  pre-processor corner (swap 2<->3,
// 6<->7), meshNekReader.cpp:30 / con.c:6
const int kPreToSymVertex[8] = {0, 1, 3, 2, 4, 5, 7, 6};
// pre-processor face -> nekRS face (t-, s-, r+, s+, r-, t+), meshNekReader.cpp:31
const int kPreToNekrsFace[6] = {1, 2, 3, 4, 0, 5};
// pre-processor face -> symmetric face, con.c:7
const int kPreToSymFace[6] = {2, 1, 3, 0, 4, 5};
// vertices (hypercube order, 1-based) of each symmetric face, con-periodic.c:3-5
const int kSymFaceVerts[6][4] = {{1, 5, 7, 3}, {2, 4, 8, 6}, {1, 2, 6, 5}, {3, 7, 8, 4}, {1, 3, 4, 2}, {5, 6, 8, 7}};
// the three edge neighbours of each hypercube vertex, con.c:8-10
const int kNeighbor[8][3] = {{1, 2, 4}, {0, 3, 5}, {0, 3, 6}, {1, 2, 7}, {0, 5, 6}, {1, 4, 7}, {2, 4, 7}, {3, 5, 6}};

struct File {
  FILE *fp = nullptr;
  std::string path;
  long long size = 0;
  explicit File(const char *p) : path(p ? p : "")
  {
    if (!p) throw Error(NRSG_ERR_INVALID, "re2: null path");
    fp = std::fopen(p, "rb");
    if (!fp) throw Error(NRSG_ERR_INVALID, "re2: cannot open " + path);
    std::fseek(fp, 0, SEEK_END);
    size = std::ftell(fp);
  }
  File(const File &) = delete;
  File &operator=(const File &) = delete;
  ~File()
  {
    if (fp) std::fclose(fp);
  }
  void read(long long off, void *dst, size_t bytes)
  {
    if (off < 0 || off + (long long)bytes > size) throw Error(NRSG_ERR_INVALID, "re2: truncated file " + path);
    std::fseek(fp, (long)off, SEEK_SET);
    if (std::fread(dst, 1, bytes, fp) != bytes) throw Error(NRSG_ERR_INVALID, "re2: read failed on " + path);
  }
};

void swap_bytes(unsigned char *p, size_t word, size_t nwords)
{
  for (size_t w = 0; w < nwords; ++w, p += word) std::reverse(p, p + word);
}

struct Layout {
  nrsg_re2_header h{};
  int wdsize = 8;
  long long curveOff = 0;               // offset of the curve count
  std::vector<long long> bcOff;         // offset of each boundary section's count
  std::vector<long long> bcCount;
};

double word_at(File &f, const Layout &L, long long off)
{
  unsigned char b[8];
  if (L.wdsize == 8) {
    f.read(off, b, 8);
    if (L.h.byteSwapped) swap_bytes(b, 8, 1);
    double d;
    std::memcpy(&d, b, 8);
    return d;
  }
  f.read(off, b, 4);
  if (L.h.byteSwapped) swap_bytes(b, 4, 1);
  float v;
  std::memcpy(&v, b, 4);
  return v;
}

Layout scan(File &f)
{
  Layout L;
  char hdr[81] = {0};
  if (f.size < 84) throw Error(NRSG_ERR_INVALID, "re2: file too short: " + f.path);
  f.read(0, hdr, 80);
  const std::string s(hdr, 80);
  const std::string ver = s.substr(0, 5);
  long long nelgt = 0, nelgv = 0, nbc = 0;
  int ndim = 0;
  if (ver == "#v004") {
    if (std::sscanf(hdr + 5, "%lld %d %lld %lld", &nelgt, &ndim, &nelgv, &nbc) < 3)
      throw Error(NRSG_ERR_INVALID, "re2: bad v004 header");
    L.h.version = 4;
  } else if (ver == "#v002" || ver == "#v003") {
    // Fortran format (a5, i9, i3, i9)
    nelgt = std::atoll(s.substr(5, 9).c_str());
    ndim = std::atoi(s.substr(14, 3).c_str());
    nelgv = std::atoll(s.substr(17, 9).c_str());
    L.h.version = ver == "#v002" ? 2 : 3;
  } else {
    throw Error(NRSG_ERR_INVALID, "re2: unsupported version '" + ver + "' (v002, v003, v004 are read)");
  }
  if (ndim != 3) throw Error(NRSG_ERR_INVALID, "re2: only 3-D meshes are supported (ndim=" + std::to_string(ndim) + ")");
  if (nelgt <= 0 || nelgv <= 0 || nelgv > nelgt) throw Error(NRSG_ERR_INVALID, "re2: invalid element counts in header");
  float test;
  f.read(80, &test, 4);
  if (test == 6.54321f) {
    L.h.byteSwapped = 0;
  } else {
    unsigned char b[4];
    std::memcpy(b, &test, 4);
    swap_bytes(b, 4, 1);
    std::memcpy(&test, b, 4);
    if (test != 6.54321f) throw Error(NRSG_ERR_INVALID, "re2: byte-order test word not found");
    L.h.byteSwapped = 1;
  }
  L.wdsize = 8;
  L.h.ndim = ndim;
  L.h.nelgt = nelgt;
  L.h.nelgv = nelgv;
  const long long recWords = 1 + 3 * 8;
  L.curveOff = 84 + nelgt * recWords * L.wdsize;
  const double nc = word_at(f, L, L.curveOff);
  L.h.ncurve = (long long)nc;
  if (L.h.ncurve < 0) throw Error(NRSG_ERR_INVALID, "re2: negative curve count");
  long long off = L.curveOff + L.wdsize + L.h.ncurve * 8 * L.wdsize;
  while (off < f.size) {
    const long long cnt = (long long)word_at(f, L, off);
    if (cnt < 0 || off + L.wdsize + cnt * 8 * L.wdsize > f.size) throw Error(NRSG_ERR_INVALID, "re2: bad boundary section");
    L.bcOff.push_back(off);
    L.bcCount.push_back(cnt);
    off += L.wdsize + cnt * 8 * L.wdsize;
  }
  if (off != f.size) throw Error(NRSG_ERR_INVALID, "re2: trailing bytes after the boundary sections");
  L.h.nbcFields = (int)L.bcOff.size();
  if (L.h.version == 4 && nbc > 0 && nbc != L.h.nbcFields)
    throw Error(NRSG_ERR_INVALID, "re2: header announces " + std::to_string(nbc) + " boundary sections, file holds " +
                                      std::to_string(L.h.nbcFields));
  return L;
}

// one 8-word record: element, face, p[5], character word
struct Record {
  long long elem;
  int face;
  double p[5];
  char code[4];
};

void read_records(File &f, const Layout &L, long long off, long long cnt, std::vector<Record> &out)
{
  out.resize(cnt);
  std::vector<unsigned char> buf(cnt * 8 * L.wdsize);
  if (cnt) f.read(off, buf.data(), buf.size());
  for (long long r = 0; r < cnt; ++r) {
    unsigned char *q = buf.data() + r * 8 * L.wdsize;
    if (L.h.byteSwapped) swap_bytes(q, 8, 7); // the character word is not swapped
    double w[7];
    std::memcpy(w, q, sizeof(w));
    Record &R = out[r];
    R.elem = (long long)w[0] - 1;
    R.face = (int)w[1] - 1;
    for (int k = 0; k < 5; ++k) R.p[k] = w[2 + k];
    std::memcpy(R.code, q + 56, 3);
    R.code[3] = 0;
    if (R.elem < 0 || R.elem >= L.h.nelgt || R.face < 0 || R.face > 5)
      throw Error(NRSG_ERR_INVALID, "re2: record with element/face out of range");
  }
}

// ---- parCon restated for one process ---------------------------------------
struct Point {
  double x[3];
  double dx;     // squared distance to the nearest edge neighbour in its element
  long long seq; // 8*element + hypercube vertex
};

// find_unique_vertices (con-unique-vertices.c:385-446) on one rank: all
// points start as one segment; ndim rounds of (sort each segment by x, y, z in
// turn; open a new segment where consecutive points differ by more than
// tol * sqrt(min(dx)) in that coordinate).  Segment order gives the ids.
void unique_vertices(std::vector<Point> &P, double tol, std::vector<long long> &gid)
{
  const size_t n = P.size();
  const double tol2 = tol * tol;
  std::vector<char> start(n, 0);
  if (n) start[0] = 1;
  for (int t = 0; t < 3; ++t)
    for (int d = 0; d < 3; ++d) {
      size_t s = 0;
      while (s < n) {
        size_t e = s + 1;
        while (e < n && !start[e]) ++e;
        // ties keep their order (the result does not depend on it for
        // vertices that coincide exactly)
        std::stable_sort(P.begin() + s, P.begin() + e, [d](const Point &a, const Point &b) { return a.x[d] < b.x[d]; });
        s = e;
      }
      for (size_t j = 1; j < n; ++j) {
        const double df = (P[j].x[d] - P[j - 1].x[d]) * (P[j].x[d] - P[j - 1].x[d]);
        if (df > std::min(P[j].dx, P[j - 1].dx) * tol2) start[j] = 1;
      }
    }
  gid.assign(n, 0);
  long long id = -1;
  for (size_t j = 0; j < n; ++j) {
    if (start[j]) ++id;
    gid[j] = id;
  }
}

long long find_root(std::vector<long long> &parent, long long a)
{
  while (parent[a] != a) a = parent[a] = parent[parent[a]];
  return a;
}

} // namespace

extern "C" {

#define RE2_TRY(...)                                                                                           \
  try {                                                                                                        \
    __VA_ARGS__;                                                                                               \
    return NRSG_OK;                                                                                            \
  } catch (const Error &e) {                                                                                   \
    nrsg::set_last_error(e.what());                                                                            \
    return e.code;                                                                                             \
  } catch (const std::bad_alloc &) {                                                                           \
    nrsg::set_last_error("host allocation failed");                                                            \
    return NRSG_ERR_OOM;                                                                                       \
  } catch (const std::exception &e) {                                                                          \
    nrsg::set_last_error(e.what());                                                                            \
    return NRSG_ERR_INVALID;                                                                                   \
  }

int nrsg_re2_read_header(const char *path, nrsg_re2_header *hdr)
{
  if (!hdr) return NRSG_ERR_INVALID;
  RE2_TRY({
    File f(path);
    *hdr = scan(f).h;
  })
}

int nrsg_re2_read_elements(const char *path, double *h_VX, int *h_group)
{
  RE2_TRY({
    File f(path);
    const Layout L = scan(f);
    const long long E = L.h.nelgt;
    const size_t rec = 25 * 8;
    const long long chunk = 65536;
    std::vector<unsigned char> buf;
    for (long long e0 = 0; e0 < E; e0 += chunk) {
      const long long ne = std::min(chunk, E - e0);
      buf.resize(ne * rec);
      f.read(84 + e0 * (long long)rec, buf.data(), buf.size());
      if (L.h.byteSwapped) swap_bytes(buf.data(), 8, ne * 25);
      for (long long i = 0; i < ne; ++i) {
        double w[25];
        std::memcpy(w, buf.data() + i * rec, sizeof(w));
        const long long e = e0 + i;
        if (h_group) h_group[e] = (int)w[0];
        if (h_VX)
          for (int v = 0; v < 8; ++v)
            for (int c = 0; c < 3; ++c) h_VX[(e * 8 + v) * 3 + c] = w[1 + 8 * c + kPreToSymVertex[v]];
      }
    }
  })
}

int nrsg_re2_read_curves(const char *path, long long *h_elem, int *h_face, double *h_params, char *h_type)
{
  RE2_TRY({
    File f(path);
    const Layout L = scan(f);
    std::vector<Record> R;
    read_records(f, L, L.curveOff + L.wdsize, L.h.ncurve, R);
    for (long long r = 0; r < L.h.ncurve; ++r) {
      if (h_elem) h_elem[r] = R[r].elem;
      if (h_face) h_face[r] = R[r].face;
      if (h_params) std::memcpy(h_params + 5 * r, R[r].p, 5 * sizeof(double));
      if (h_type) h_type[r] = R[r].code[0];
    }
  })
}

int nrsg_re2_read_bc(const char *path, int field, char *h_cbc, double *h_bc)
{
  RE2_TRY({
    File f(path);
    const Layout L = scan(f);
    if (field < 0 || field >= L.h.nbcFields)
      throw Error(NRSG_ERR_INVALID, "re2: boundary section " + std::to_string(field) + " not in file (" +
                                        std::to_string(L.h.nbcFields) + " sections)");
    const long long E = L.h.nelgt;
    if (h_cbc)
      for (long long i = 0; i < E * 6; ++i) std::memcpy(h_cbc + 4 * i, "E  ", 4);
    if (h_bc) std::fill(h_bc, h_bc + E * 30, 0.0);
    std::vector<Record> R;
    read_records(f, L, L.bcOff[field] + L.wdsize, L.bcCount[field], R);
    for (const Record &r : R) {
      const long long k = r.elem * 6 + r.face;
      if (h_cbc) std::memcpy(h_cbc + 4 * k, r.code, 4);
      if (h_bc) std::memcpy(h_bc + 5 * k, r.p, 5 * sizeof(double));
    }
  })
}

int nrsg_re2_boundary_ids(long long E, const char *h_cbc, int ncodes, const char *const *codes, const int *ids,
                          int *h_EToB)
{
  if (E < 1 || !h_cbc || ncodes < 0 || (ncodes && (!codes || !ids)) || !h_EToB) return NRSG_ERR_INVALID;
  RE2_TRY({
    std::vector<std::string> key(ncodes);
    for (int k = 0; k < ncodes; ++k) {
      std::string c = codes[k] ? codes[k] : "";
      if (c.size() > 3) throw Error(NRSG_ERR_INVALID, "re2: boundary codes have at most 3 characters");
      c.resize(3, ' ');
      key[k] = c;
    }
    for (long long e = 0; e < E; ++e)
      for (int f = 0; f < 6; ++f) {
        const std::string c(h_cbc + 4 * (e * 6 + f), 3);
        int id = 0;
        for (int k = 0; k < ncodes; ++k)
          if (c == key[k]) { id = ids[k]; break; }
        h_EToB[e * 6 + kPreToNekrsFace[f]] = id;
      }
  })
}

int nrsg_mesh_connect(long long E, const double *h_VX, double tol, const char *h_cbc, const double *h_bc,
                      long long *h_EToV, long long *nvertices)
{
  if (E < 1 || !h_VX || !h_EToV || !(tol > 0)) return NRSG_ERR_INVALID;
  RE2_TRY({
    const size_t n = (size_t)E * 8;
    std::vector<Point> P(n);
    for (long long e = 0; e < E; ++e)
      for (int v = 0; v < 8; ++v) {
        Point &p = P[e * 8 + v];
        for (int c = 0; c < 3; ++c) p.x[c] = h_VX[(e * 8 + v) * 3 + c];
        p.seq = e * 8 + v;
      }
    // findMinNeighborDistance (con.c:85-117)
    for (long long e = 0; e < E; ++e)
      for (int v = 0; v < 8; ++v) {
        Point &p = P[e * 8 + v];
        double m = 1.7976931348623157e308;
        for (int k = 0; k < 3; ++k) {
          const Point &q = P[e * 8 + kNeighbor[v][k]];
          const double d = (p.x[0] - q.x[0]) * (p.x[0] - q.x[0]) + (p.x[1] - q.x[1]) * (p.x[1] - q.x[1]) +
                           (p.x[2] - q.x[2]) * (p.x[2] - q.x[2]);
          m = std::min(m, d);
        }
        p.dx = m;
      }
    std::vector<Point> S = P;
    std::vector<long long> segId;
    unique_vertices(S, tol, segId);
    std::vector<long long> gid(n);
    for (size_t j = 0; j < n; ++j) gid[S[j].seq] = segId[j];

    // periodic faces (matchPeriodicFaces, con-periodic.c:266-281)
    if (h_cbc && h_bc) {
      struct Face {
        long long e;
        int f, cf;
        long long ce;
      };
      std::vector<Face> F;
      for (long long e = 0; e < E; ++e)
        for (int f = 0; f < 6; ++f)
          if (std::strncmp(h_cbc + 4 * (e * 6 + f), "P  ", 3) == 0) {
            const double *b = h_bc + 5 * (e * 6 + f);
            const long long ce = (long long)b[0] - 1;
            const int cf = (int)b[1] - 1;
            if (ce < 0 || ce >= E || cf < 0 || cf > 5) throw Error(NRSG_ERR_INVALID, "re2: periodic face links out of range");
            F.push_back({e, kPreToSymFace[f], kPreToSymFace[cf], ce});
          }
      // union ids (component minimum) over matched vertex pairs
      std::vector<long long> idRoot(n);
      std::iota(idRoot.begin(), idRoot.end(), 0LL);
      for (size_t i = 0; i < F.size(); ++i)
        for (size_t j = i + 1; j < F.size(); ++j) {
          if (!(F[j].ce == F[i].e && F[j].cf == F[i].f)) continue;
          // findConnectedPeriodicPairs (con-periodic.c:117-178)
          double fx[4][3], gx[4][3];
          long long fid[4], gidv[4];
          double fMax = 0, gMax = 0;
          for (int j2 = 0; j2 < 4; ++j2) {
            const long long pf = F[i].e * 8 + kSymFaceVerts[F[i].f][j2] - 1;
            const long long pg = F[j].e * 8 + kSymFaceVerts[F[j].f][j2] - 1;
            for (int c = 0; c < 3; ++c) {
              fx[j2][c] = P[pf].x[c];
              gx[j2][c] = P[pg].x[c];
            }
            fid[j2] = gid[pf];
            gidv[j2] = gid[pg];
          }
          for (int c = 0; c < 3; ++c) {
            double mf = 0, mg = 0;
            for (int j2 = 0; j2 < 4; ++j2) {
              fMax = std::max(fMax, std::fabs(fx[j2][c]));
              gMax = std::max(gMax, std::fabs(gx[j2][c]));
              mf += fx[j2][c];
              mg += gx[j2][c];
            }
            for (int j2 = 0; j2 < 4; ++j2) {
              fx[j2][c] -= mf / 4;
              gx[j2][c] -= mg / 4;
            }
          }
          int shift = 0;
          double d2Min = 1e20;
          for (int s = 0; s < 4; ++s) {
            double d2 = 0;
            for (int j2 = 0; j2 < 4; ++j2) {
              const int k = 3 - (j2 + s) % 4;
              for (int c = 0; c < 3; ++c) d2 += (fx[j2][c] - gx[k][c]) * (fx[j2][c] - gx[k][c]);
            }
            if (d2 < d2Min) { d2Min = d2; shift = s; }
          }
          if (std::sqrt(d2Min) > 1e-3 * std::max(fMax, gMax))
            throw Error(NRSG_ERR_INVALID, "re2: periodic faces do not match (element " + std::to_string(F[i].e + 1) + ")");
          for (int j2 = 0; j2 < 4; ++j2) {
            const int k = 3 - (j2 + shift) % 4;
            const long long a = find_root(idRoot, fid[j2]), b = find_root(idRoot, gidv[k]);
            if (a != b) idRoot[std::max(a, b)] = std::min(a, b);
          }
        }
      for (size_t p = 0; p < n; ++p) gid[p] = find_root(idRoot, gid[p]);
    }
    // compressPeriodicVertices (con-periodic.c:17-50): consecutive ids in id order
    std::vector<long long> sorted(gid);
    std::sort(sorted.begin(), sorted.end());
    sorted.erase(std::unique(sorted.begin(), sorted.end()), sorted.end());
    for (size_t p = 0; p < n; ++p) h_EToV[p] = 1 + (std::lower_bound(sorted.begin(), sorted.end(), gid[p]) - sorted.begin());
    if (nvertices) *nvertices = (long long)sorted.size();
  })
}

} // extern "C"
