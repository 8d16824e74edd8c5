"""Oracle package (test infrastructure only): the C++ restatement of parry3d and its ctypes wrapper."""
