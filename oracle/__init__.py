"""CPU oracle of FJSPH's hot path (test infrastructure only; see oracle.cpp)."""
