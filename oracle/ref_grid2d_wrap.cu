// C entry points over the reference's own grid2D host/device index functions
// (simplex/src/common_cpx/form01mapping.cu:4-57), compiled from the reference sources
// where they lie by oracle/ref_build.sh into oracle/_ref/libref_grid2d.so. TEST
// INFRASTRUCTURE ONLY: used to pin the 2D oracle's blocked layout. No kernel is launched.
#include "form01mapping.h"

extern "C" {
static grid2D mk(int n) {
    grid2D g;
    g.init(n, n);
    return g;
}
int ref2_cell_size(int n) { return mk(n).cell_size(); }
int ref2_face_size(int n, int d) { return mk(n).face_size(d); }
int ref2_node_size(int n) { return mk(n).node_size(); }
int ref2_cell_ind(int n, int x, int y) { return mk(n).cell_ind(x, y); }
int ref2_face_ind(int n, int x, int y, int d) { return mk(n).face_ind(x, y, d); }
int ref2_node_ind(int n, int x, int y) { return mk(n).node_ind(x, y); }
void ref2_ind_cell(int n, int i, int* xy) { mk(n).ind_cell(i, xy[0], xy[1]); }
}
