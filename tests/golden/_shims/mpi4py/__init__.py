"""Single-rank stand-in for mpi4py, used only to import the reference package in
the container that generates golden fixtures (mpi4py is not installed there)."""
