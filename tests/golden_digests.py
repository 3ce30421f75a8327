"""Digests of seeded synthetic workloads, fixed so that a host whose generator
drifts (e.g. a different platform) fails loudly instead of benchmarking other jobs."""
SYNTH_EXT2_2000_SEED11 = "f61ab3f469cf06f3"
