// ghosts.cuh -- ghost cells of boundp and bounduvw as compositions of maps.
//
// set_bc (src/bound.f90:227-646) runs three passes over the whole extended
// faces, x then y then z (boundp: src/bound.f90:146-225, bounduvw: 17-144).
// Every pass reads only cells that no pass writes (interior cells next to the
// boundary), so the final value of a written cell is a composition of at most
// three maps, one per direction, each acting on one cell of its line:
// unchanged, a copy, F + S*v, or a constant F.  This header builds the maps of
// every written position on the host by replaying the passes' writes (the last
// write of a position wins) and evaluates the composition of one cell, with the
// passes' arithmetic (F + S*v with S in {-1, 0, 1}: an exact product, one
// rounding), so the values are bit-identical to running the three passes.
// k_ghosts (kernels.cuh) evaluates every written cell in one launch; the CPU
// emulator (emu.cu) runs the same code for the tests.
#pragma once

#ifndef FG_HD
#define FG_HD __host__ __device__ __forceinline__
#endif

namespace fg {

enum : int { GM_KEEP = 0, GM_COPY = 1, GM_AFF = 2, GM_CONST = 3 };
struct GMap {
  double F, S;
  int src, kind;
};
constexpr int GM_SLOTS = 9;  // 2h + 1, h <= 4: slot -t for t <= 0, h + t - n for t >= n
template <int NC> struct GhostArgs {
  double *f[NC];
  int n[3], h;
  int hi[3];  // positions 1..hi[d] are never written (hi = n or n - 1)
  GMap m[NC][3][GM_SLOTS];
};

// One side of one direction of bounduvw for one component (k_set_bc3's form).
struct BcSide {
  char ctype;
  int centered;
  double factor[4];
  double sgn;
};

inline int gm_slot(int t, int n, int h) { return t <= 0 ? -t : h + t - n; }
inline void gm_set(GMap *m, int n, int h, int t, int kind, int src, double F = 0.0, double S = 0.0) {
  m[gm_slot(t, n, h)] = GMap{F, S, src, kind};
}
inline void gm_clear(GMap *m) {
  for (int s = 0; s < GM_SLOTS; s++) m[s] = GMap{0.0, 0.0, 0, GM_KEEP};
}
// True when no map of the line reads a position the line writes (the maps
// then compose; grids too small for it keep the pass-by-pass kernels).
inline bool gm_closed(const GMap *m, int n, int h) {
  for (int s = 0; s < 2 * h + 1; s++) {
    if (m[s].kind != GM_COPY && m[s].kind != GM_AFF) continue;
    const int t = m[s].src;
    if (t < 1 || t > n || (t == n && m[h].kind != GM_KEEP)) return false;
  }
  return true;
}

// boundp's maps (centred set_bc, nh_p = 1): periodic copies, and
// ghost = f + s * inner (D: f = 2 bc, s = -1; N: f = -+dr bc, s = 1).  Every
// field of a gets the same maps.
template <int NC>
inline void boundp_maps(GhostArgs<NC> &a, const int n[3], const char cbc[6], const double bc[6],
                        const double dr[3][2]) {
  auto fs = [&](char ct, int ib, double rv, double drv, double *f, double *sc) {
    if (ct == 'D') { *f = 2.0 * rv; *sc = -1.0; }
    else if (ct == 'N') { *f = ib == 0 ? -drv * rv : drv * rv; *sc = 1.0; }
    else { *f = 0.0; *sc = 0.0; }
  };
  a.h = 1;
  for (int d = 0; d < 3; d++) {
    a.n[d] = n[d];
    GMap *m = a.m[0][d];
    gm_clear(m);
    double f, sc;
    if (cbc[2 * d] == 'P') gm_set(m, n[d], 1, 0, GM_COPY, n[d]);
    else { fs(cbc[2 * d], 0, bc[2 * d], dr[d][0], &f, &sc); gm_set(m, n[d], 1, 0, GM_AFF, 1, f, sc); }
    if (cbc[2 * d + 1] == 'P') gm_set(m, n[d], 1, n[d] + 1, GM_COPY, 1);
    else { fs(cbc[2 * d + 1], 1, bc[2 * d + 1], dr[d][1], &f, &sc); gm_set(m, n[d], 1, n[d] + 1, GM_AFF, n[d], f, sc); }
    for (int c = 1; c < NC; c++)
      for (int sl = 0; sl < GM_SLOTS; sl++) a.m[c][d][sl] = m[sl];
  }
}

// The sides of bounduvw's passes (src/bound.f90:17-144): cbc, bc in Fortran
// (0:1,1:3,1:3) order; dzc_h, dzf_h host arrays (1-nh_d:nz+nh_d).
inline void setbc_sides(const char *cbc, const double *bc, int nz, int nh_d, int h, const double dl[3],
                        const double *dzc_h, const double *dzf_h, BcSide side[3][3][2]) {
  for (int d = 0; d < 3; d++)
    for (int c = 0; c < 3; c++)
      for (int ib = 0; ib < 2; ib++) {
        BcSide &sd = side[d][c][ib];
        sd.ctype = cbc[ib + 2 * d + 6 * c];
        sd.centered = (c != d) ? 1 : 0;  // the face-normal component is not centred
        double dr[4];
        for (int q = 0; q < h; q++) {
          if (d < 2) dr[q] = dl[d];
          else if (c < 2) dr[q] = ib == 0 ? dzc_h[-q - 1 + nh_d] : dzc_h[nz + q - 1 + nh_d];
          else dr[q] = ib == 0 ? dzf_h[-q - 1 + nh_d] : dzf_h[nz + q - 1 + nh_d];
        }
        const double rv = bc[ib + 2 * d + 6 * c];
        sd.sgn = 0.0;
        for (int q = 0; q < h; q++) sd.factor[q] = rv;
        if (sd.ctype == 'D' && sd.centered) { for (int q = 0; q < h; q++) sd.factor[q] = 2.0 * rv; sd.sgn = -1.0; }
        if (sd.ctype == 'N') {
          for (int q = 0; q < h; q++) sd.factor[q] = ib == 0 ? -dr[q] * rv : dr[q] * rv;
          sd.sgn = 1.0;
        }
      }
}

// The maps of one direction and component of bounduvw's set_bc pass
// (both ends, layers in order, the last write of a cell wins).
inline void setbc_maps(GMap *m, const BcSide side[2], int n, int h) {
  gm_clear(m);
  for (int ib = 0; ib < 2; ib++) {
    const BcSide &sd = side[ib];
    for (int q = 0; q < h; q++) {
      const double f = sd.factor[q];
      if (sd.ctype == 'P') {
        gm_set(m, n, h, 0 - q, GM_COPY, n - q);
        gm_set(m, n, h, n + 1 + q, GM_COPY, 1 + q);
      } else if (sd.centered) {
        if (ib == 0) gm_set(m, n, h, 0 - q, GM_AFF, 1 + q, f, sd.sgn);
        else gm_set(m, n, h, n + 1 + q, GM_AFF, n - q, f, sd.sgn);
      } else if (sd.ctype == 'D') {
        if (ib == 0) {
          gm_set(m, n, h, 0 - q, GM_CONST, 0, f);
        } else {
          gm_set(m, n, h, n + q, GM_CONST, 0, f);
          gm_set(m, n, h, n + 1 + q, GM_COPY, n - 1 - q);
        }
      } else {
        if (ib == 0) {
          gm_set(m, n, h, 0 - q, GM_AFF, 1 + q, 1.0 * f, 1.0);
        } else {
          gm_set(m, n, h, n + q, GM_AFF, n - 1 - q, 1.0 * f, 1.0);
          gm_set(m, n, h, n + 1 + q, GM_AFF, n - 1 - q, 2.0 * f, 1.0);
        }
      }
    }
  }
}

// Completes a (hi) and tells whether the maps compose; *count: the written cells.
template <int NC> inline bool ghosts_ready(GhostArgs<NC> &a, long *count) {
  for (int d = 0; d < 3; d++) {
    if (a.n[d] < 2 * a.h + 1) return false;
    a.hi[d] = a.n[d];
    for (int c = 0; c < NC; c++) {
      if (!gm_closed(a.m[c][d], a.n[d], a.h)) return false;
      if (a.m[c][d][a.h].kind != GM_KEEP) a.hi[d] = a.n[d] - 1;
    }
  }
  long E[3], w[3];
  for (int d = 0; d < 3; d++) {
    E[d] = a.n[d] + 2 * a.h;
    w[d] = E[d] - a.hi[d];
  }
  *count = w[0] * E[1] * E[2] + (long)a.hi[0] * w[1] * E[2] + (long)a.hi[0] * a.hi[1] * w[2];
  return true;
}

// The written cell of index t (x faces, then y faces without x ghosts, then z
// faces without either), 1-based coordinates in ip.
template <int NC> FG_HD void ghost_cell(const GhostArgs<NC> &a, long t, int ip[3]) {
  const int h = a.h;
  const long E0 = a.n[0] + 2 * h, E1 = a.n[1] + 2 * h, E2 = a.n[2] + 2 * h;
  const long w0 = E0 - a.hi[0], w1 = E1 - a.hi[1];
  const long c0 = a.hi[0], c1 = a.hi[1];
  const long T0 = w0 * E1 * E2, T1 = c0 * w1 * E2;
  auto wpos = [&](int d, long s) -> int { return s < h ? (int)s + 1 - h : a.hi[d] + 1 + (int)(s - h); };
  if (t < T0) {
    ip[0] = wpos(0, t % w0);
    const long r = t / w0;
    ip[1] = (int)(r % E1) + 1 - h;
    ip[2] = (int)(r / E1) + 1 - h;
  } else if (t < T0 + T1) {
    const long u = t - T0;
    ip[0] = (int)(u % c0) + 1;
    const long r = u / c0;
    ip[1] = wpos(1, r % w1);
    ip[2] = (int)(r / w1) + 1 - h;
  } else {
    const long u = t - T0 - T1;
    ip[0] = (int)(u % c0) + 1;
    const long r = u / c0;
    ip[1] = (int)(r % c1) + 1;
    ip[2] = wpos(2, r / c1);
  }
}

// Up to four ranges of the enumeration above: the written cells whose z
// position lies in a range of planes (x faces, y faces, low and high z faces
// of those planes), for the ghost cells of a z-slab of the field.
struct GhostSegs {
  long begin[4], count[4];
  int n;
  long total;
};
FG_HD long ghost_seg_cell(const GhostSegs &s, long q) {
  int r = 0;
  while (r < s.n - 1 && q >= s.count[r]) q -= s.count[r++];
  return s.begin[r] + q;
}
// The segments of extended z planes [e0, e1) (plane e = z position - 1 + h);
// a.hi must be set (ghosts_ready).
template <int NC> inline GhostSegs ghost_segs_of_planes(const GhostArgs<NC> &a, int e0, int e1) {
  const int h = a.h;
  const long E0 = a.n[0] + 2 * h, E1 = a.n[1] + 2 * h, E2 = a.n[2] + 2 * h;
  const long w0 = E0 - a.hi[0], w1 = E1 - a.hi[1], w2 = E2 - a.hi[2];
  const long c0 = a.hi[0], c1 = a.hi[1];
  const long T0 = w0 * E1 * E2, T1 = c0 * w1 * E2;
  GhostSegs s{};
  auto add = [&](long b, long c) {
    if (c <= 0) return;
    s.begin[s.n] = b;
    s.count[s.n] = c;
    s.n++;
    s.total += c;
  };
  add(w0 * E1 * e0, w0 * E1 * (e1 - e0));             // x faces of the planes
  add(T0 + c0 * w1 * e0, c0 * w1 * (e1 - e0));        // y faces
  long lo = e0 > 0 ? e0 : 0, hi = e1 < h ? e1 : h;    // low z faces: slot s at plane s
  add(T0 + T1 + c0 * c1 * lo, c0 * c1 * (hi - lo));
  lo = e0 - a.hi[2] > h ? e0 - a.hi[2] : h;           // high z faces: slot s at plane hi[2] + s
  hi = e1 - a.hi[2] < w2 ? e1 - a.hi[2] : w2;
  add(T0 + T1 + c0 * c1 * lo, c0 * c1 * (hi - lo));
  if (s.n == 0) s.n = 1;  // empty: one segment of no cells
  return s;
}

// The final value of field c at the written cell ip; false when the cell is
// unchanged for that field (nothing to write).  The x map applies first.
template <int NC> FG_HD bool ghost_value(const GhostArgs<NC> &a, int c, const int ip[3], double *out) {
  const int h = a.h;
  const long E0 = a.n[0] + 2 * h, E1 = a.n[1] + 2 * h;
  const GMap *mp[3];
  bool any = false;
  for (int d = 0; d < 3; d++) {
    const int tt = ip[d];
    mp[d] = (tt <= 0 || tt > a.hi[d]) ? &a.m[c][d][tt <= 0 ? -tt : h + tt - a.n[d]] : nullptr;
    if (mp[d] && mp[d]->kind == GM_KEEP) mp[d] = nullptr;
    any |= mp[d] != nullptr;
  }
  if (!any) return false;
  // sources, z map first; a constant ends the chain
  int sp[3] = {ip[0], ip[1], ip[2]};
  int top = -1;  // the direction whose constant starts the chain (-1: a cell of the field)
  for (int d = 2; d >= 0; d--) {
    if (!mp[d]) continue;
    if (mp[d]->kind == GM_CONST) { top = d; break; }
    sp[d] = mp[d]->src;
  }
  double v;
  int from;
  if (top >= 0) {
    v = mp[top]->F;
    from = top + 1;
  } else {
    v = a.f[c][(long)(sp[0] - 1 + h) + E0 * ((long)(sp[1] - 1 + h) + E1 * (long)(sp[2] - 1 + h))];
    from = 0;
  }
  for (int d = from; d < 3; d++)
    if (mp[d] && mp[d]->kind == GM_AFF) v = mp[d]->F + mp[d]->S * v;
  *out = v;
  return true;
}

template <int NC> FG_HD long ghost_index(const GhostArgs<NC> &a, const int ip[3]) {
  const int h = a.h;
  const long E0 = a.n[0] + 2 * h, E1 = a.n[1] + 2 * h;
  return (long)(ip[0] - 1 + h) + E0 * ((long)(ip[1] - 1 + h) + E1 * (long)(ip[2] - 1 + h));
}

}  // namespace fg
