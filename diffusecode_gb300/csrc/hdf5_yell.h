// The output menu's HDF5 ("Yell 1.0") file, written without an HDF5 library.
#pragma once
#include "../../include/discus_gpu.h"

namespace dgpu_hdf5 {

// gen_hdf5_write's file for the values v (qval over out_inc, i fastest):
// DGPU_OK or DGPU_ERR_IO.
int write_yell(const char *path, const dgpu_output *o, const double *v);

}  // namespace dgpu_hdf5
