// SAMRAI configuration stand-in (no MPI, no HDF5).
