"""mlff_gb300 -- GB300-native energy/force/MD path of a PaiNN-style
StudentForceField (drop-in for MLFF-Distiller's model, ASE calculator and
velocity-Verlet NVE loop)."""
__version__ = "0.1.0"
