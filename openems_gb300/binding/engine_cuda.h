/*
 * engine_cuda.h -- the openEMS-side binding of the GB300 engine (`--engine=cuda`).
 *
 * These two classes are what a maintainer adds to openEMS's FDTD/ directory next to the
 * basic/sse/sse-compressed/multithreaded engines (openems.h:161-166, openems.cpp:221-265,
 * openems.cpp:725-755):
 *
 *   - Operator_CUDA derives from Operator_SSE_Compressed (FDTD/operator_sse_compressed.h), so the
 *     whole coefficient build and CompressOperator run unchanged; only CreateEngine() differs,
 *     following FDTD/operator_sse_compressed.cpp:46-54.
 *   - Engine_CUDA derives from Engine (FDTD/engine.h) and forwards its interface to the C ABI of
 *     include/oems_cuda.h.  Instead of creating CPU engine extensions (Engine::InitExtensions,
 *     FDTD/engine.cpp:61-73) it hands each Operator_Ext_*'s built tables to the device engine.
 *
 * The operator-extension tables are protected members.  The binding reads them through member
 * pointers formed in small accessor subclasses (engine_cuda.cpp), so it compiles against the
 * reference headers unchanged; a maintainer may equally add one `friend class Engine_CUDA;` line
 * per operator-extension header.  tests/test_binding_builds.py compiles and links this file
 * against the reference's own headers and objects.
 */
#ifndef OEMS_ENGINE_CUDA_H
#define OEMS_ENGINE_CUDA_H

#include <stdexcept>
#include <string>
#include <vector>

#include "FDTD/engine.h"
#include "FDTD/operator_sse_compressed.h"
#include "oems_cuda.h"

class Engine_CUDA;

class Operator_CUDA : public Operator_SSE_Compressed
{
public:
	static Operator_CUDA* New();
	Engine* CreateEngine() override;

protected:
	Operator_CUDA() : Operator_SSE_Compressed() {}
};

class Engine_CUDA : public Engine
{
public:
	static Engine_CUDA* New(const Operator_CUDA* op, int device = 0);
	~Engine_CUDA() override;

	void Init() override;
	void Reset() override;
	//! allocate the device step state for up to maxTS steps; openEMS::RunFDTD calls it before
	//! its first IterateTS (probes register through the C ABI before it)
	void StartRun(unsigned int maxTS);
	bool IterateTS(unsigned int iterTS) override;
	unsigned int GetNumberOfTimesteps() override;

	FDTD_FLOAT GetVolt(unsigned int n, unsigned int x, unsigned int y, unsigned int z) const override;
	FDTD_FLOAT GetVolt(unsigned int n, const unsigned int pos[3]) const override;
	FDTD_FLOAT GetCurr(unsigned int n, unsigned int x, unsigned int y, unsigned int z) const override;
	FDTD_FLOAT GetCurr(unsigned int n, const unsigned int pos[3]) const override;
	void SetVolt(unsigned int n, unsigned int x, unsigned int y, unsigned int z, FDTD_FLOAT value) override;
	void SetVolt(unsigned int n, const unsigned int pos[3], FDTD_FLOAT value) override;
	void SetCurr(unsigned int n, unsigned int x, unsigned int y, unsigned int z, FDTD_FLOAT value) override;
	void SetCurr(unsigned int n, const unsigned int pos[3], FDTD_FLOAT value) override;

	//! the device engine, for the probe/dump registration of the processing layer
	oems_cuda_engine* Handle() const { return m_h; }

protected:
	Engine_CUDA(const Operator_CUDA* op, int device);
	void Check(int rc, const char* what) const;

	const Operator_CUDA* m_OpCUDA;
	int m_device;
	oems_cuda_engine* m_h;
	bool m_started;
};

#endif
