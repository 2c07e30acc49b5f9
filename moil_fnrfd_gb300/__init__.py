"""GB300-native MOIL nonbonded energy/force path (cutoff LJ + real-space Ewald,
PME reciprocal sum, pair-list rebuild) behind MOIL's eforce()/COMMON interface."""
