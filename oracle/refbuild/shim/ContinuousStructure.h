/*
 * ORACLE BUILD SHIM -- test infrastructure only.
 *
 * Declaration-only stand-in for CSXCAD's headers (ContinuousStructure.h, CSPrim*.h, CSProp*.h,
 * CSRectGrid.h).  CSXCAD is a separate, un-vendored project; it is not installed in this image.
 * The openEMS translation units compiled by oracle/refbuild/build_ref.py include it only for the
 * operator's geometry and material lookups, which the harness never calls: the harness fills the
 * operator coefficients and extension tables itself.  Every member function here therefore aborts
 * with its name if it is ever reached.  Enum values are this shim's own (distinct bits); no code
 * path that the harness runs compares them.
 */
#ifndef OEMS_SHIM_CONTINUOUSSTRUCTURE_H
#define OEMS_SHIM_CONTINUOUSSTRUCTURE_H

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

[[noreturn]] inline void oems_shim_unreachable(const char* what)
{
	std::fprintf(stderr, "openEMS oracle harness: CSXCAD stand-in '%s' was called\n", what);
	std::abort();
}
#define OEMS_SHIM_ABORT { oems_shim_unreachable(__PRETTY_FUNCTION__); }

enum CoordinateSystem { CARTESIAN = 0, CYLINDRICAL = 1, UNDEFINED_CS = 2 };

inline void Point_Line_Distance(const double*, const double*, const double*, double&, double&,
                                CoordinateSystem = CARTESIAN) OEMS_SHIM_ABORT
inline std::string ConvertInt(int) OEMS_SHIM_ABORT
inline void TransformCoordSystem(const double*, double*, CoordinateSystem, CoordinateSystem) OEMS_SHIM_ABORT

class CSPrimitives;
class CSPrimBox;
class CSPrimCurve;
class CSPropMaterial;
class CSPropLumpedElement;
class CSPropExcitation;
class CSPropLorentzMaterial;
class CSPropDebyeMaterial;
class CSPropConductingSheet;
class CSPropAbsorbingBC;
class CSFunctionParser;

class CSProperties
{
public:
	enum PropertyType
	{
		ANY = 0x7fffffff, UNKNOWN = 0x1, MATERIAL = 0x2, METAL = 0x4, EXCITATION = 0x8,
		PROBEBOX = 0x10, RESBOX = 0x20, DUMPBOX = 0x40, DISPERSIVEMATERIAL = 0x80,
		LORENTZMATERIAL = 0x100, DEBYEMATERIAL = 0x200, DISCRETE_MATERIAL = 0x400,
		LUMPED_ELEMENT = 0x800, CONDUCTINGSHEET = 0x1000, ABSORBING_BC = 0x2000
	};
	virtual ~CSProperties() {}
	PropertyType GetType() const OEMS_SHIM_ABORT
	std::string GetName() const OEMS_SHIM_ABORT
	unsigned int GetID() const OEMS_SHIM_ABORT
	size_t GetQtyPrimitives() const OEMS_SHIM_ABORT
	CSPrimitives* GetPrimitive(size_t) OEMS_SHIM_ABORT
	std::vector<CSPrimitives*> GetAllPrimitives() OEMS_SHIM_ABORT
	CSPropMaterial* ToMaterial() OEMS_SHIM_ABORT
	CSPropLumpedElement* ToLumpedElement() OEMS_SHIM_ABORT
	CSPropExcitation* ToExcitation() OEMS_SHIM_ABORT
	CSPropConductingSheet* ToConductingSheet() OEMS_SHIM_ABORT
	CSPropLorentzMaterial* ToLorentzMaterial() OEMS_SHIM_ABORT
	CSPropDebyeMaterial* ToDebyeMaterial() OEMS_SHIM_ABORT
	bool GetVisibility() const OEMS_SHIM_ABORT
	std::string GetAttributeValue(const std::string&) const OEMS_SHIM_ABORT
	bool ExistAttribute(const std::string&) const OEMS_SHIM_ABORT
};

class ParameterCoord
{
public:
	double* GetCoords(CoordinateSystem) OEMS_SHIM_ABORT
	double GetCoordValue(int, CoordinateSystem) OEMS_SHIM_ABORT
};

class CSPrimitives
{
public:
	virtual ~CSPrimitives() {}
	unsigned int GetID() const OEMS_SHIM_ABORT
	std::string GetTypeName() const OEMS_SHIM_ABORT
	int GetPriority() const OEMS_SHIM_ABORT
	CSProperties* GetProperty() const OEMS_SHIM_ABORT
	bool GetBoundBox(double*, bool = false) OEMS_SHIM_ABORT
	int GetDimension() OEMS_SHIM_ABORT
	bool IsInside(const double*, double = 0) OEMS_SHIM_ABORT
	void SetPrimitiveUsed(bool) OEMS_SHIM_ABORT
	bool GetPrimitiveUsed() const OEMS_SHIM_ABORT
	CSPrimBox* ToBox() OEMS_SHIM_ABORT
	CSPrimCurve* ToCurve() OEMS_SHIM_ABORT
	CoordinateSystem GetCoordinateSystem() const OEMS_SHIM_ABORT
	CoordinateSystem GetBoundBoxCoordSystem() const OEMS_SHIM_ABORT
};

class CSPrimBox : public CSPrimitives
{
public:
	ParameterCoord* GetStartCoord() OEMS_SHIM_ABORT
	ParameterCoord* GetStopCoord() OEMS_SHIM_ABORT
};

class CSPrimCurve : public CSPrimitives
{
public:
	size_t GetNumberOfPoints() OEMS_SHIM_ABORT
	bool GetPoint(size_t, double*, CoordinateSystem = UNDEFINED_CS, bool = false) OEMS_SHIM_ABORT
};

class CSPropMaterial : public CSProperties
{
public:
	double GetEpsilonWeighted(int, const double*) OEMS_SHIM_ABORT
	double GetKappaWeighted(int, const double*) OEMS_SHIM_ABORT
	double GetMueWeighted(int, const double*) OEMS_SHIM_ABORT
	double GetSigmaWeighted(int, const double*) OEMS_SHIM_ABORT
	double GetDensityWeighted(const double*) OEMS_SHIM_ABORT
	double GetEpsilon(int = 0) OEMS_SHIM_ABORT
	double GetMue(int = 0) OEMS_SHIM_ABORT
	double GetKappa(int = 0) OEMS_SHIM_ABORT
	double GetSigma(int = 0) OEMS_SHIM_ABORT
	bool GetIsotropy() OEMS_SHIM_ABORT
};

class CSBackgroundMaterial
{
public:
	double GetEpsilon() OEMS_SHIM_ABORT
	double GetMue() OEMS_SHIM_ABORT
	double GetKappa() OEMS_SHIM_ABORT
	double GetSigma() OEMS_SHIM_ABORT
};

class CSPropLumpedElement : public CSProperties
{
public:
	enum LEtype { INVALID = -1, PARALLEL = 0, SERIES = 1 };
	double GetCapacity() const OEMS_SHIM_ABORT
	double GetResistance() const OEMS_SHIM_ABORT
	double GetInductance() const OEMS_SHIM_ABORT
	int GetDirection() const OEMS_SHIM_ABORT
	bool GetCaps() const OEMS_SHIM_ABORT
	LEtype GetLEtype() const OEMS_SHIM_ABORT
};

class CSPropExcitation : public CSProperties
{
public:
	int GetExcitType() const OEMS_SHIM_ABORT
	double GetExcitation(int, int = 0) OEMS_SHIM_ABORT
	double GetWeightedExcitation(int, const double*) OEMS_SHIM_ABORT
	bool GetActiveDir(int) OEMS_SHIM_ABORT
	double GetDelay() OEMS_SHIM_ABORT
	double GetFrequency() OEMS_SHIM_ABORT
	double* GetPropagationDir() OEMS_SHIM_ABORT
	unsigned int GetNumber() OEMS_SHIM_ABORT
	bool GetEnabled() const OEMS_SHIM_ABORT
};

class CSPropDiscMaterial : public CSPropMaterial {};

class CSPropDispersiveMaterial : public CSPropMaterial
{
public:
	int GetDispersionOrder() OEMS_SHIM_ABORT
};

class CSPropLorentzMaterial : public CSPropDispersiveMaterial
{
public:
	double GetEpsPlasmaFreqWeighted(int, int, const double*) OEMS_SHIM_ABORT
	double GetMuePlasmaFreqWeighted(int, int, const double*) OEMS_SHIM_ABORT
	double GetEpsLorPoleFreqWeighted(int, int, const double*) OEMS_SHIM_ABORT
	double GetMueLorPoleFreqWeighted(int, int, const double*) OEMS_SHIM_ABORT
	double GetEpsRelaxTimeWeighted(int, int, const double*) OEMS_SHIM_ABORT
	double GetMueRelaxTimeWeighted(int, int, const double*) OEMS_SHIM_ABORT
};

class CSPropDebyeMaterial : public CSPropDispersiveMaterial
{
public:
	double GetEpsDeltaWeighted(int, int, const double*) OEMS_SHIM_ABORT
	double GetEpsRelaxTimeWeighted(int, int, const double*) OEMS_SHIM_ABORT
};

class CSPropConductingSheet : public CSPropMaterial
{
public:
	double GetConductivity() OEMS_SHIM_ABORT
	double GetThickness() OEMS_SHIM_ABORT
};

class CSPropAbsorbingBC : public CSProperties {};

class CSRectGrid
{
public:
	static CSRectGrid* Clone(CSRectGrid*) OEMS_SHIM_ABORT
	double* GetLines(int, double*, unsigned int&, bool = false) OEMS_SHIM_ABORT
	double GetDeltaUnit() OEMS_SHIM_ABORT
	CoordinateSystem GetMeshType() OEMS_SHIM_ABORT
	double GetLine(int, size_t) OEMS_SHIM_ABORT
	void SetLine(int, size_t, double) OEMS_SHIM_ABORT
	void AddDiscLine(int, double) OEMS_SHIM_ABORT
	void ClearLines(int, bool = false) OEMS_SHIM_ABORT
};

class ContinuousStructure
{
public:
	CSBackgroundMaterial* GetBackgroundMaterial() OEMS_SHIM_ABORT
	CSRectGrid* GetGrid() OEMS_SHIM_ABORT
	CSProperties* GetPropertyByCoordPriority(const double*, std::vector<CSPrimitives*>, bool = false,
	                                         CSPrimitives** = NULL) OEMS_SHIM_ABORT
	CSProperties* GetPropertyByCoordPriority(const double*, CSProperties::PropertyType = CSProperties::ANY,
	                                         bool = false, CSPrimitives** = NULL) OEMS_SHIM_ABORT
	std::vector<CSProperties*> GetPropertyByType(CSProperties::PropertyType) OEMS_SHIM_ABORT
	std::vector<CSPrimitives*> GetPrimitivesByBoundBox(const double*, bool = false,
	                                                   CSProperties::PropertyType = CSProperties::ANY) OEMS_SHIM_ABORT
	std::vector<CSPrimitives*> GetAllPrimitives(bool = false, CSProperties::PropertyType = CSProperties::ANY) OEMS_SHIM_ABORT
	std::vector<CSPrimitives*> GetPrimitivesByType(int) OEMS_SHIM_ABORT
	size_t GetQtyProperties() OEMS_SHIM_ABORT
	CSProperties* GetProperty(size_t) OEMS_SHIM_ABORT
	CSFunctionParser* GetFunctionParser() OEMS_SHIM_ABORT
};

#endif
