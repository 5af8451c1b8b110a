"""Physical <-> lattice unit conversion (mirrors src/lbm/units.mojo:91-210)."""
from __future__ import annotations


class Unit:
    """One quantity with its physical and lattice value."""

    def __init__(self, physical: float, lattice: float):
        self.physical = float(physical)
        self.lattice = float(lattice)

    def C_phys_to_lat(self) -> float:
        return self.lattice / self.physical

    def C_lat_to_phys(self) -> float:
        return self.physical / self.lattice


class UnitSystem:
    """Velocity, length, time and density scales; tau = 3 nu_lat + 0.5 (units.mojo:115-128)."""

    def __init__(self, u_physical: float, u_lattice: float, L_physical: float, L_lattice: float,
                 density: float, kinematic_viscosity: float, D: int = 3):
        self.D = D
        self.U = Unit(u_physical, u_lattice)
        self.L = Unit(L_physical, L_lattice)
        self.t = Unit((L_physical / u_physical) / (L_lattice / u_lattice), 1.0)
        self.density = Unit(density, 1.0)
        self.Re = (self.U.physical * self.L.physical) / kinematic_viscosity
        v_lat = self.U.lattice * self.L.lattice / self.Re
        self.dt = self.t.physical
        self.tau = v_lat / (1 / 3.0) + 0.5
        self.kinematic_viscosity = Unit(kinematic_viscosity, v_lat)
        self.mass = Unit(self.density.C_lat_to_phys() * (self.L.C_lat_to_phys() ** D), 1.0)
        self.force = Unit(self.density.C_lat_to_phys() * self.L.C_lat_to_phys() ** (D - 1)
                          * self.U.C_lat_to_phys() ** 2, 1.0)
        self.pressure = Unit(self.force.C_lat_to_phys() / self.L.C_lat_to_phys() ** (D - 1), 1.0)


def tau_from_Re(u_lattice: float, L_lattice: float, Re: float) -> float:
    """tau = 3 u L / Re + 0.5 (units.mojo:123-126)."""
    return 3.0 * u_lattice * L_lattice / Re + 0.5
