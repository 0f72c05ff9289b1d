"""CPU oracle of the docking energy path -- test infrastructure only (see oracle.h)."""
