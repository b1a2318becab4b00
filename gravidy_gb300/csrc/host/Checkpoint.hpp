// Exact checkpoints of a run (the format of gravidy_gb300/checkpoint.py):
// magic "H4CHK001", u64 n, 14 f64 scalars, then r[n][4], v[n][4], f[n][6],
// t[n], dt[n] (f64) and ids[n] (u32), little endian.  The reference resumes
// from 4-digit ASCII snapshots and recomputes forces and timesteps
// (src/include/utils/OptionsParser.cpp:122-323); resuming from a checkpoint
// continues the run bit for bit.
#ifndef GRAVIDY_GB300_HOST_CHECKPOINT_HPP
#define GRAVIDY_GB300_HOST_CHECKPOINT_HPP

#include <string>

#include "NbodySystem.hpp"

namespace gb300 {

struct CheckpointScalars {
    double e2, eta, dt_min, dt_max, itime, atime, iterations, nsteps, interactions, e_ini, e_tmp, output_factor,
        snapshot_number, t_end;
};

// Writes the NbodySystem arrays (h_r, h_v, h_f, h_t, h_dt, h_id).
bool write_checkpoint(const std::string &path, const NbodySystem &ns, const CheckpointScalars &sc);
// Reads a checkpoint into ns (allocating its arrays); n and e2/eta are set.
bool read_checkpoint(const std::string &path, NbodySystem &ns, CheckpointScalars &sc);

}  // namespace gb300
#endif
