"""GB300-native vortex-filament velocity and time-step path (OpenVort drop-in)."""
