"""GB300-native (sm_103a) time step of the wPFAW3D phase-field acid-wormholing model."""
