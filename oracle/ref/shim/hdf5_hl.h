/* See hdf5.h in this directory: no-op stand-in for the HDF5 high-level API. */
#include "hdf5.h"
