"""GB300-native continuous max-flow (ASETS) solvers."""
