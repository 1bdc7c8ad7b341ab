// C entry points over the reference's own grid3D host/device index functions
// (simplex/src/common_cpx/grid3D.cu:24-146), compiled from the reference sources where
// they lie by oracle/ref_build.sh into oracle/_ref/libref_grid3d.so. TEST
// INFRASTRUCTURE ONLY: used to pin the oracle's blocked layout. No kernel is launched.
#include "grid3D.h"

extern "C" {
int ref_cell_size(int n) { return grid3D(n, n, n).cell_size(); }
int ref_face_size(int n, int d) { return grid3D(n, n, n).face_size(d); }
int ref_edge_size(int n, int d) { return grid3D(n, n, n).edge_size(d); }
int ref_cell_ind(int n, int x, int y, int z) { return grid3D(n, n, n).cell_ind(x, y, z); }
int ref_face_ind(int n, int x, int y, int z, int d) { return grid3D(n, n, n).face_ind(x, y, z, d); }
int ref_edge_ind(int n, int x, int y, int z, int d) { return grid3D(n, n, n).edge_ind(x, y, z, d); }
void ref_ind_cell(int n, int i, int* xyz) { grid3D(n, n, n).ind_cell(i, xyz[0], xyz[1], xyz[2]); }
void ref_ind_face(int n, int i, int d, int* xyz) { grid3D(n, n, n).ind_face(i, d, xyz[0], xyz[1], xyz[2]); }
int ref_face_valid(int n, int x, int y, int z, int d) { return grid3D(n, n, n).face_valid(x, y, z, d) ? 1 : 0; }
}
