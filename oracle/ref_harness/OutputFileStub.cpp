// Oracle-build replacement for the reference's OutputFile.cpp, which needs VTK.
// The harness writes its own binary dumps; the reference's periodic
// WriteOutput (Simulation.cpp:872-876) becomes a no-op here.
#include "OutputFile.h"

OutputFile::OutputFile(int outputIdx) : m_outputIdx(outputIdx) {}
OutputFile::~OutputFile() {}
void OutputFile::WriteVTK_LocalData(SubDomain&) {}
void OutputFile::WriteVTK_Collective(SubDomain&) {}
void OutputFile::WriteSurfaceAttribute(SubDomain&, int) {}
