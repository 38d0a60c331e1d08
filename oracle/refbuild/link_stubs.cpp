/*
 * link_stubs.cpp -- ORACLE BUILD, test infrastructure only.
 *
 * Link-time stand-ins for the two openEMS definitions whose translation units are not compiled
 * into the harness, because they need libraries that are not installed in this image:
 *   - tools/global.cpp (Boost.Program_options): the global settings object g_settings, with the
 *     default state its constructor sets (verbose level 0, no native dumps);
 *   - tools/vtk_file_writer.cpp (VTK): VTK_File_Writer, used only by the operator's debug dumps,
 *     which the harness never writes; every member aborts if reached.
 */
#include <cstdio>
#include <cstdlib>

#include "tools/global.h"
#include "tools/vtk_file_writer.h"

Global g_settings;

Global::Global()
{
	m_showProbeDiscretization = false;
	m_nativeFieldDumps = false;
	m_VerboseLevel = 0;
	m_SavedVerboseLevel = 0;
	m_optionDesc = NULL;
}

[[noreturn]] static void vtk_unreachable(const char* what)
{
	std::fprintf(stderr, "openEMS oracle harness: VTK_File_Writer stand-in '%s' was called\n", what);
	std::abort();
}

VTK_File_Writer::VTK_File_Writer(std::string, int) { vtk_unreachable(__func__); }
VTK_File_Writer::~VTK_File_Writer() {}
void VTK_File_Writer::SetMeshLines(double const* const*, unsigned int const*, double) { vtk_unreachable(__func__); }
void VTK_File_Writer::AddScalarField(std::string, double const* const* const*) { vtk_unreachable(__func__); }
void VTK_File_Writer::AddScalarField(std::string, float const* const* const*) { vtk_unreachable(__func__); }
void VTK_File_Writer::AddVectorField(std::string, double const* const* const* const*) { vtk_unreachable(__func__); }
void VTK_File_Writer::AddVectorField(std::string, float const* const* const* const*) { vtk_unreachable(__func__); }
void VTK_File_Writer::AddVectorField(std::string, ArrayLib::ArrayNIJK<float>&) { vtk_unreachable(__func__); }
int VTK_File_Writer::GetNumberOfFields() const { vtk_unreachable(__func__); }
void VTK_File_Writer::ClearAllFields() { vtk_unreachable(__func__); }
bool VTK_File_Writer::Write() { vtk_unreachable(__func__); }
bool VTK_File_Writer::WriteASCII() { vtk_unreachable(__func__); }
bool VTK_File_Writer::WriteXML() { vtk_unreachable(__func__); }
std::string VTK_File_Writer::GetTimestepFilename(int) const { vtk_unreachable(__func__); }
