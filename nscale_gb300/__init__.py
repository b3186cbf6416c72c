"""nscale_gb300 — GB300-native (sm_103a) nuclei-segmentation hot path of nscale."""
