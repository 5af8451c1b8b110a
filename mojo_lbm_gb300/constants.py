"""Constants of the LBM step: flags, streaming methods, collision operators
(mirrors src/lbm/constants.mojo:10-136)."""
from __future__ import annotations

cs = (1.0 / 3.0) ** 0.5
cs_squared = 1.0 / 3.0


class LBM_method:
    """Streaming methods (constants.mojo:20-31)."""
    DOUBLE_BUFFER = 0
    ESOTERIC_PULL = 1
    valid_set = {DOUBLE_BUFFER, ESOTERIC_PULL}


DOUBLE_BUFFER = LBM_method.DOUBLE_BUFFER
ESOTERIC_PULL = LBM_method.ESOTERIC_PULL


class Collisions:
    """Collision operator names (constants.mojo:41-55) and their C-ABI ids."""
    SRT = "SRT"
    TRT = "TRT"
    KBC = "KBC"
    RLBM = "RLBM"
    valid_set = {SRT, TRT, KBC, RLBM}
    that_need_fneq = {KBC, RLBM}
    ids = {SRT: 0, TRT: 1, KBC: 2, RLBM: 3}


class Flags:
    """Node flags (constants.mojo:58-116): a low-nibble enum plus high-bit masks."""
    FLUID = 0
    SOLID = 1
    EQUILIBRIUM = 2
    FLUID_SOLID_BOUNDARY = 3
    EXCLUDE = 0b10000000
    CAPTURE_DENSITY = 0b01000000
    CAPTURE_VELOCITY = 0b00100000
    valid_enums = {FLUID, SOLID, EQUILIBRIUM, FLUID_SOLID_BOUNDARY}
    valid_bitmasks = {EXCLUDE, CAPTURE_DENSITY, CAPTURE_VELOCITY}

    @staticmethod
    def get_enum_flag(flag: int) -> int:
        return flag & 0x0F

    @staticmethod
    def get_bitmask_flags(flag: int) -> int:
        return flag >> 4

    @staticmethod
    def is_(enum_flag: int, flag: int) -> bool:
        if enum_flag not in Flags.valid_enums:
            raise ValueError(f"{enum_flag} is not a flag enum")
        return (flag & 0x0F) == enum_flag

    @staticmethod
    def has(bitmask_flag: int, flag: int) -> bool:
        if bitmask_flag not in Flags.valid_bitmasks:
            raise ValueError(f"{bitmask_flag} is not a flag bitmask")
        return (bitmask_flag & flag) != 0

    @staticmethod
    def add_exclude_to_flag(flag: int) -> int:
        return Flags.EXCLUDE | flag

    @staticmethod
    def is_excluded(flag: int) -> bool:
        return bool(Flags.EXCLUDE & flag)


class Bounceback_method:
    """Bounce-back variants (constants.mojo:120-123)."""
    MID_GRID = 0
    BOUZIDI = 1


FLUID_NODE = Flags.FLUID
SOLID_NODE = Flags.SOLID
