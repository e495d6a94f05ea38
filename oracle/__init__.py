"""ORACLE — TEST INFRASTRUCTURE ONLY (CPU restatement of the reference; see hsr_oracle.cpp)."""
