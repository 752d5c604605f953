"""ORACLE -- test infrastructure only: a CPU restatement of the reference's flood-engine
time step used to check the CUDA path.  The product package never imports it."""
