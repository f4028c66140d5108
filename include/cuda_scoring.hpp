// The reference's scoring-backend selector interface (include/cuda_scoring.hpp
// of githubofzby/beam, C++ linkage). libbeam_gb300.so exports both functions
// with these exact signatures: CudaScoringBuildMode() returns "cuda" and
// CudaScoringCompiled() returns true, so a reference build linking this
// library instead of src/cuda_scoring_stub.cpp reports the CUDA backend
// (printed at src/main.cpp:504).
#pragma once

const char* CudaScoringBuildMode();
bool CudaScoringCompiled();
