/*
 * plt_writer.h -- host half of the snapshot writers (MPM::Output_plt_file,
 * mpm_ini.cpp:832-980): the Tecplot binary header of the particle file and the
 * ASCII cell table.  The context (capi.cu) packs the data on the device and
 * copies it out; these functions only lay out bytes and text.
 */
#pragma once
#include <cstdint>
#include <string>

namespace pgdg_out {

/* the particle file up to its data: "#!TDV112", one ordered zone "grid" of n
 * points, the twelve variables x y z phase vx vy vol rho P tv v n_neighbor
 * (doubles, with phase and n_neighbor as int32), the solution time, and the
 * placeholder ranges (-1, 1) the reference writes for every variable */
std::string plt_header(int64_t n, double time);

/* the cell table: two header lines, then one line per cell in lexicographic
 * order (i outer, then j, then k): the centre (box_l + (i + 1/2) p_size per
 * axis, 0 beyond the dimension) and the twelve packed columns (cols[12 c ..]),
 * each value as an ostream writes a double by default (printf %g), separated
 * and ended by a space.  Formatted on `threads` host threads.  Returns 0, or -1
 * with msg set. */
int write_cell_table(const char* path, int dim, const int N[3], const double box_l[3], const double p_size[3],
                     const double* cols, double time, int threads, std::string* msg);

}  // namespace pgdg_out
