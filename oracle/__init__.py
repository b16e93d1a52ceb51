"""CPU oracle of the AeroApps aerosol-optics + VLIDORT path (test infrastructure only)."""
