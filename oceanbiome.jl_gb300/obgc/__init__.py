"""obgc — GB300-native OceanBioME tracer-tendency engine (Python side of the C ABI)."""
