"""zeno_gb300: GB300-native CUDA state-vector backend for zeno."""
