"""GB300-native free-wake unsteady vortex-lattice engine (VOLCANOR hot path)."""
