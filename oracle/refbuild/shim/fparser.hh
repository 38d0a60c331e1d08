/*
 * ORACLE BUILD SHIM -- test infrastructure only.  Declaration-only stand-in for fparser (not
 * installed in this image).  openEMS uses it for custom excitation signals and for the UPML
 * grading string while the operator is built; the harness builds neither (it is given the
 * signal and the UPML tables).  Parse() only records the expression and reports success (-1,
 * fparser's "no error" result), because Operator_Ext_UPML's constructor parses its default grading
 * string; every member that would evaluate an expression aborts if reached.
 */
#ifndef OEMS_SHIM_FPARSER_HH
#define OEMS_SHIM_FPARSER_HH
#include <string>
#include "ContinuousStructure.h"
class FunctionParser
{
public:
	enum ParseErrorType { SYNTAX_ERROR = 0, FP_NO_ERROR = 1 };
	bool AddConstant(const std::string&, double) OEMS_SHIM_ABORT
	int Parse(const std::string& expr, const std::string&, bool = false)
	{
		m_expr = expr;
		return -1;
	}
	ParseErrorType GetParseErrorType() const OEMS_SHIM_ABORT
	const char* ErrorMsg() const OEMS_SHIM_ABORT
	double Eval(const double*) OEMS_SHIM_ABORT
	int EvalError() const OEMS_SHIM_ABORT

private:
	std::string m_expr;
};
#endif
