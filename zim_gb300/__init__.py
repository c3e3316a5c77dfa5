"""zim_gb300: GB300-native structured-light stereo reconstruction path."""
