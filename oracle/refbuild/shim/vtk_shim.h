/*
 * ORACLE BUILD SHIM -- test infrastructure only.  Declaration-only stand-in for the few VTK
 * classes that openEMS's Operator uses in its debug dumps (DumpPEC2File and friends).  VTK is not
 * installed in this image and the harness never writes those dumps.
 */
#ifndef OEMS_SHIM_VTK_H
#define OEMS_SHIM_VTK_H
#include "ContinuousStructure.h"
#define VTK_MAJOR_VERSION 9
typedef long long vtkIdType;
class vtkPoints { public: static vtkPoints* New() OEMS_SHIM_ABORT
	vtkIdType InsertNextPoint(const double*) OEMS_SHIM_ABORT
	vtkIdType InsertNextPoint(double, double, double) OEMS_SHIM_ABORT
	void Delete() OEMS_SHIM_ABORT };
class vtkCellArray { public: static vtkCellArray* New() OEMS_SHIM_ABORT
	vtkIdType InsertNextCell(int) OEMS_SHIM_ABORT
	void InsertCellPoint(vtkIdType) OEMS_SHIM_ABORT
	void Delete() OEMS_SHIM_ABORT };
class vtkPolyData { public: static vtkPolyData* New() OEMS_SHIM_ABORT
	void SetPoints(vtkPoints*) OEMS_SHIM_ABORT
	void SetLines(vtkCellArray*) OEMS_SHIM_ABORT
	void Delete() OEMS_SHIM_ABORT };
class vtkXMLPolyDataWriter { public: static vtkXMLPolyDataWriter* New() OEMS_SHIM_ABORT
	void SetInputData(vtkPolyData*) OEMS_SHIM_ABORT
	void SetFileName(const char*) OEMS_SHIM_ABORT
	int Write() OEMS_SHIM_ABORT
	void Delete() OEMS_SHIM_ABORT };
#endif
