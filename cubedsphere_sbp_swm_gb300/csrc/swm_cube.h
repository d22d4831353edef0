// swm_cube.h -- cube topology on the host: panel frames and the index map of
// a panel's points into the unfolded frame of a neighbouring panel.
//
// Follows transform_index / find_basis_orientation of the reference
// (topology/cubed_sphere_topology_mod.f90:80-239): panel p has the frame
// (ex, ey, n) and integer origin r; a point (is, js) of source panel ps lands
// at (it, jt) of target panel pt's frame extended across their common edge,
// with nx x ny points per panel row / column of the target's point type.
#pragma once

namespace swm {
namespace cube {

inline constexpr int kEX[6][3] = {{-1, 0, 0}, {0, 0, -1}, {1, 0, 0}, {0, 0, 1}, {1, 0, 0}, {1, 0, 0}};
inline constexpr int kEY[6][3] = {{0, 1, 0}, {0, 1, 0}, {0, 1, 0}, {0, 1, 0}, {0, 0, 1}, {0, 0, -1}};
inline constexpr int kN[6][3] = {{0, 0, 1}, {-1, 0, 0}, {0, 0, -1}, {1, 0, 0}, {0, 1, 0}, {0, -1, 0}};
inline constexpr int kR[6][3] = {{1, 0, 0}, {1, 0, 1}, {0, 0, 1}, {0, 0, 0}, {0, 0, 0}, {0, 1, 1}};

inline int dot3(const int* a, const int* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// frame of target panel pt unfolded across its edge with source panel ps
inline void unfolded_frame(int ps, int pt, int nx, int ny, int exl[3], int eyl[3], int rl[3], int sh[2]) {
  const int dr = dot3(kEX[pt], kN[ps]), db = dot3(kEY[pt], kN[ps]);
  for (int c = 0; c < 3; ++c) {
    if (dr == -1) { exl[c] = kN[pt][c]; eyl[c] = kEY[pt][c]; rl[c] = kR[pt][c] + kEX[pt][c]; }
    else if (dr == 1) { exl[c] = -kN[pt][c]; eyl[c] = kEY[pt][c]; rl[c] = kR[pt][c] + kN[pt][c]; }
    else if (db == 1) { exl[c] = kEX[pt][c]; eyl[c] = -kN[pt][c]; rl[c] = kR[pt][c] + kN[pt][c]; }
    else if (db == -1) { exl[c] = kEX[pt][c]; eyl[c] = kN[pt][c]; rl[c] = kR[pt][c] + kEY[pt][c]; }
    else { exl[c] = -kEX[pt][c]; eyl[c] = kEY[pt][c]; rl[c] = kR[pt][c] + kEX[pt][c] + kN[pt][c]; }
  }
  if (dr == -1) { sh[0] = nx; sh[1] = 0; }
  else if (dr == 1) { sh[0] = -nx; sh[1] = 0; }
  else if (db == 1) { sh[0] = 0; sh[1] = -ny; }
  else if (db == -1) { sh[0] = 0; sh[1] = ny; }
  else { sh[0] = 2 * nx; sh[1] = 0; }
}

// 1-based point (is, js) of panel ps -> 1-based (possibly halo) index of pt
inline void map_index(int ps, int is, int js, int pt, int nx, int ny, int& it, int& jt) {
  if (ps == pt) { it = is; jt = js; return; }
  int exl[3], eyl[3], rl[3], sh[2], d[3];
  unfolded_frame(ps, pt, nx, ny, exl, eyl, rl, sh);
  for (int c = 0; c < 3; ++c) d[c] = kR[ps][c] - rl[c];
  it = (is - 1) * dot3(kEX[ps], exl) + (js - 1) * dot3(kEY[ps], exl) + (nx - 1) * dot3(d, exl) + 1 + sh[0];
  jt = (is - 1) * dot3(kEX[ps], eyl) + (js - 1) * dot3(kEY[ps], eyl) + (ny - 1) * dot3(d, eyl) + 1 + sh[1];
}

// find_basis_orientation(ps, pt): whether the two frames keep their axes
// (dim_i) and the directions of the sender's loops, which are also the signs
// of the vector components the halo exchange packs.
inline void orientation(int ps, int pt, int& istep, int& jstep, int& dim_i) {
  if (ps == pt) { istep = 1; jstep = 1; dim_i = 1; return; }
  int exl[3], eyl[3], rl[3], sh[2];
  unfolded_frame(ps, pt, 2, 2, exl, eyl, rl, sh);
  const int ex_ex = dot3(kEX[ps], exl), ex_ey = dot3(kEY[ps], exl);
  const int ey_ex = dot3(kEX[ps], eyl), ey_ey = dot3(kEY[ps], eyl);
  if (ex_ex != 0) { dim_i = 1; istep = ex_ex; jstep = ey_ey; }
  else { dim_i = 0; istep = ex_ey; jstep = ey_ex; }
}

}  // namespace cube
}  // namespace swm
