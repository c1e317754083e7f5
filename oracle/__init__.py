"""FP64 CPU oracle of the projector -- test infrastructure only (see oracle.cpp)."""
