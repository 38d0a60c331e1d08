/*
 * harness.cpp -- ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * Drives openEMS's own engine, compiled unmodified from the reference sources by
 * oracle/refbuild/build_ref.py, through the same C ABI shape as include/oems_cuda.h (prefix
 * oems_refeng_).  The tests use it to pin the C restatement (oracle/oems_oracle.c), the host
 * operator tables (openems_gb300/operator.py) and, through fixtures it generates, the CUDA engine.
 * bench.py times it as the reference's CPU engine.  Nothing in the product links it.
 *
 * What runs is the reference's code:
 *   - the engines Engine (FDTD/engine.cpp), Engine_sse, Engine_SSE_Compressed and
 *     Engine_Multithread (FDTD/engine_multithread.cpp, its x-slab worker threads and barriers);
 *   - Operator_SSE_Compressed::CompressOperator (FDTD/operator_sse_compressed.cpp:114-175);
 *   - the engine extensions Engine_Ext_Excitation, _UPML, _Mur_ABC, _LorentzMaterial and their
 *     priority sort (FDTD/engine.cpp:87-98);
 *   - the probes ProcessVoltage / ProcessCurrent through ProcessIntegral::Process
 *     (Common/processintegral.cpp:134-171), with Engine_Interface_FDTD's integrals and
 *     CalcFastEnergy;
 *   - the excitation signal Excitation::buildExcitationSignal (FDTD/excitation.cpp:95-176).
 *
 * What the harness supplies instead of CSXCAD (which is not available): the operator
 * coefficients and the operator-extension tables, written into the reference's own members by
 * small subclasses (the same values Operator::CalcECOperator and each BuildExtension would
 * store), and the extension insertion order of openEMS::SetupFDTD (openems.cpp:1186-1241,
 * 383-407): excitation, Mur walls, UPML regions, Lorentz/Drude.  The processing loop follows
 * openEMS::RunFDTD: probes run once before the first step and after every chunk of steps, the
 * chunk being the smallest next interval the probes report (ProcessingArray::Process).
 *
 * Every entry point restores the caller's floating-point environment on return.  The reference's
 * SSE engines set flush-to-zero on x86 (Denormal::Disable, tools/denormal.h); that state is kept
 * per engine and applied only while the engine computes, so the calling process is unaffected.
 */
#include <cfenv>
#include <climits>
#include <cstdint>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "FDTD/engine.h"
#include "FDTD/engine_interface_fdtd.h"
#include "FDTD/engine_multithread.h"
#include "FDTD/engine_sse.h"
#include "FDTD/engine_sse_compressed.h"
#include "FDTD/excitation.h"
#include "FDTD/extensions/operator_ext_excitation.h"
#include "FDTD/extensions/operator_ext_lorentzmaterial.h"
#include "FDTD/extensions/operator_ext_mur_abc.h"
#include "FDTD/extensions/operator_ext_upml.h"
#include "FDTD/operator.h"
#include "FDTD/operator_multithread.h"
#include "FDTD/operator_sse.h"
#include "FDTD/operator_sse_compressed.h"
#include "Common/processcurrent.h"
#include "Common/processvoltage.h"

namespace {

enum { OK = 0, ERR_ARG = 1, ERR_STATE = 3, ERR_UNSUPPORTED = 4, ERR_NOMEM = 6 };
enum { KIND_BASIC = 0, KIND_SSE = 1, KIND_SSE_COMPRESSED = 2, KIND_MULTITHREAD = 3 };

/* ---------------------------------------------------------------------------------------- */
/* operator: the reference's class with the members CalcECOperator would fill set directly     */

template <class Base>
class HOp : public Base
{
public:
	HOp() : Base() { this->Init(); }

	void SetMesh(const unsigned nl[3], const double* lines, double unit, double dt)
	{
		size_t off = 0;
		for (int n = 0; n < 3; ++n) {
			this->numLines[n] = nl[n];
			delete[] this->discLines[n];
			this->discLines[n] = new double[nl[n]];
			for (unsigned k = 0; k < nl[n]; ++k)
				this->discLines[n][k] = lines ? lines[off + k] : (double)k;
			off += nl[n];
		}
		this->gridDelta = unit;
		this->dT = dt;
	}
	void AllocCoefficients() { this->InitOperator(); }
	void SetEngine(Engine* e) { this->m_Engine = e; }
	void ForgetEngine() { this->m_Engine = NULL; }
};

/* Operator_SSE_Compressed::CalcECOperator stores CompressOperator()'s result in the protected
 * m_Use_Compression flag; the harness does the same after writing the coefficients. */
class HOpC : public HOp<Operator_SSE_Compressed>
{
public:
	bool Compress()
	{
		m_Use_Compression = false;
		m_Use_Compression = CompressOperator();
		return m_Use_Compression;
	}
	size_t Classes() const { return f4_vv_Compressed[0].size(); }
};

class HOpMT : public HOp<Operator_Multithread>
{
public:
	void ThreadLines(unsigned& t, std::vector<unsigned int>& a, std::vector<unsigned int>& b) const
	{
		CalcStartStopLines(t, a, b);
	}
	bool Compress()
	{
		m_Use_Compression = false;
		m_Use_Compression = CompressOperator();
		return m_Use_Compression;
	}
	size_t Classes() const { return f4_vv_Compressed[0].size(); }
};

/* ---------------------------------------------------------------------------------------- */
/* excitation signal and operator extensions                                                */

class HExcitation : public Excitation
{
public:
	/* given arrays (a signal type the harness does not build); period in whole steps, with the
	 * signal's own timestep set to 1 so that the engine's period/timestep is exactly that count */
	void Inject(const float* v, const float* c, unsigned len, unsigned period_steps)
	{
		Reset(0);
		Length = len;
		Signal_volt = new FDTD_FLOAT[len ? len : 1];
		Signal_curr = new FDTD_FLOAT[len ? len : 1];
		for (unsigned n = 0; n < len; ++n) {
			Signal_volt[n] = v[n];
			Signal_curr[n] = c[n];
		}
		if (period_steps) {
			dT = 1.0;
			m_SignalPeriod = (double)period_steps;
		} else {
			m_SignalPeriod = 0;
		}
	}
};

class HExtExcitation : public Operator_Ext_Excitation
{
public:
	explicit HExtExcitation(Operator* op) : Operator_Ext_Excitation(op) {}
	void Fill(Excitation* exc, unsigned nV, const unsigned* vidx, const unsigned short* vdir, const float* vamp,
	          const unsigned* vdel, unsigned nI, const unsigned* cidx, const unsigned short* cdir,
	          const float* camp, const unsigned* cdel)
	{
		m_Exc = exc;
		std::vector<unsigned int> idx[3], del, dir;
		std::vector<FDTD_FLOAT> amp;
		for (int n = 0; n < 3; ++n)
			idx[n].assign(vidx + (size_t)n * nV, vidx + (size_t)(n + 1) * nV);
		amp.assign(vamp, vamp + nV);
		del.assign(vdel, vdel + nV);
		dir.assign(vdir, vdir + nV);
		setupVoltageExcitation(idx, amp, del, dir);
		for (int n = 0; n < 3; ++n)
			idx[n].assign(cidx + (size_t)n * nI, cidx + (size_t)(n + 1) * nI);
		amp.assign(camp, camp + nI);
		del.assign(cdel, cdel + nI);
		dir.assign(cdir, cdir + nI);
		setupCurrentExcitation(idx, amp, del, dir);
	}
};

class HExtUPML : public Operator_Ext_UPML
{
public:
	explicit HExtUPML(Operator* op) : Operator_Ext_UPML(op) {}
	void Fill(const unsigned start[3], const unsigned nl[3], const float* const tab[6])
	{
		for (int n = 0; n < 3; ++n) {
			m_StartPos[n] = start[n];
			m_numLines[n] = nl[n];
		}
		ArrayLib::ArrayNIJK<FDTD_FLOAT>* arr[6] = {&vv, &vvfo, &vvfn, &ii, &iifo, &iifn};
		const char* names[6] = {"vv", "vvfo", "vvfn", "ii", "iifo", "iifn"};
		for (int a = 0; a < 6; ++a) {
			arr[a]->Init(names[a], m_numLines);
			size_t k = 0;
			for (unsigned n = 0; n < 3; ++n)
				for (unsigned x = 0; x < nl[0]; ++x)
					for (unsigned y = 0; y < nl[1]; ++y)
						for (unsigned z = 0; z < nl[2]; ++z)
							(*arr[a])(n, x, y, z) = tab[a][k++];
		}
	}
};

class HExtMur : public Operator_Ext_Mur_ABC
{
public:
	explicit HExtMur(Operator* op) : Operator_Ext_Mur_ABC(op) {}
	/* SetDirection as openems.cpp:396 calls it (top = the wall at the last line), then the
	 * coefficient planes BuildExtension would compute ([nP line][nPP line]) */
	bool Fill(int ny, unsigned line_nr, const float* cP, const float* cPP)
	{
		SetDirection(ny, line_nr != 0);
		if ((unsigned)m_LineNr != line_nr)
			return false;
		size_t k = 0;
		for (unsigned a = 0; a < m_numLines[0]; ++a)
			for (unsigned b = 0; b < m_numLines[1]; ++b, ++k) {
				m_Mur_Coeff_nyP(a, b) = cP[k];
				m_Mur_Coeff_nyPP(a, b) = cPP[k];
			}
		return true;
	}
	int LineShift() const { return m_LineNr_Shift; }
};

struct LorOrder {
	std::vector<unsigned> pos; /* [3][M] */
	bool von, con, vlon, clon;
	std::vector<float> t[6];   /* v_int, v_ext, v_lor, i_int, i_ext, i_lor: [3][M] */
};

class HExtLorentz : public Operator_Ext_LorentzMaterial
{
public:
	explicit HExtLorentz(Operator* op) : Operator_Ext_LorentzMaterial(op) {}
	/* the arrays BuildExtension allocates (operator_ext_lorentzmaterial.cpp), laid out as its
	 * destructor frees them */
	void Fill(const std::vector<LorOrder>& ords)
	{
		int order = (int)ords.size();
		m_Order = order;
		m_LM_Count.clear();
		m_LM_pos = new unsigned int**[order];
		m_volt_ADE_On = new bool[order];
		m_curr_ADE_On = new bool[order];
		m_volt_Lor_ADE_On = new bool[order];
		m_curr_Lor_ADE_On = new bool[order];
		v_int_ADE = new FDTD_FLOAT**[order];
		v_ext_ADE = new FDTD_FLOAT**[order];
		i_int_ADE = new FDTD_FLOAT**[order];
		i_ext_ADE = new FDTD_FLOAT**[order];
		v_Lor_ADE = new FDTD_FLOAT**[order];
		i_Lor_ADE = new FDTD_FLOAT**[order];
		for (int o = 0; o < order; ++o) {
			const LorOrder& L = ords[o];
			size_t M = L.pos.size() / 3;
			m_LM_Count.push_back((unsigned)M);
			m_LM_pos[o] = new unsigned int*[3];
			for (int n = 0; n < 3; ++n) {
				m_LM_pos[o][n] = new unsigned int[M ? M : 1];
				for (size_t i = 0; i < M; ++i)
					m_LM_pos[o][n][i] = L.pos[n * M + i];
			}
			m_volt_ADE_On[o] = L.von;
			m_curr_ADE_On[o] = L.con;
			m_volt_Lor_ADE_On[o] = L.vlon;
			m_curr_Lor_ADE_On[o] = L.clon;
			FDTD_FLOAT*** dst[6] = {v_int_ADE, v_ext_ADE, v_Lor_ADE, i_int_ADE, i_ext_ADE, i_Lor_ADE};
			bool on[6] = {L.von, L.von, L.vlon, L.con, L.con, L.clon};
			for (int a = 0; a < 6; ++a) {
				if (!on[a]) {
					dst[a][o] = NULL;
					continue;
				}
				dst[a][o] = new FDTD_FLOAT*[3];
				for (int n = 0; n < 3; ++n) {
					dst[a][o][n] = new FDTD_FLOAT[M ? M : 1];
					for (size_t i = 0; i < M; ++i)
						dst[a][o][n][i] = L.t[a][n * M + i];
				}
			}
		}
	}
};

/* ---------------------------------------------------------------------------------------- */
/* probes: the reference's ProcessVoltage / ProcessCurrent with the snapped box set directly  */

struct ProbeDef {
	int type; /* 0 voltage, 1 current */
	unsigned start[3], stop[3];
	int norm_dir;
	int si[3], ei[3];
	double weight;
	unsigned interval, start_ts, stop_ts;
	unsigned fd_interval;
	std::vector<double> freqs;
};

template <class P>
class HProbe : public P
{
public:
	HProbe(Engine_Interface_Base* eif, const ProbeDef& d, const std::string& name) : P(eif)
	{
		for (int n = 0; n < 3; ++n) {
			this->start[n] = d.start[n];
			this->stop[n] = d.stop[n];
			this->m_start_inside[n] = d.si[n] != 0;
			this->m_stop_inside[n] = d.ei[n] != 0;
		}
		this->m_normDir = d.norm_dir;
		this->m_dualTime = d.type == 1; /* openems.cpp:561-565: current probes use the dual time */
		this->SetWeight(d.weight);
		this->SetProcessInterval(d.interval);
		this->startTS = d.start_ts;
		this->stopTS = d.stop_ts;
		/* openems.cpp:568-571: Processing::AddFrequency derives the DFT interval from the signal's
		 * Nyquist number and each frequency; with an injected signal (no Nyquist number) the
		 * given interval is used */
		if (d.fd_interval && !d.freqs.empty()) {
			for (double f : d.freqs)
				this->AddFrequency(f);
			if (this->m_FD_Interval == 0)
				this->m_FD_Interval = d.fd_interval;
		}
		this->SetName(name);
		this->SetPrecision(17);
		this->InitProcess();
	}
	/* one ProcessIntegral::Process(); the time-domain row it writes is value*weight at slot ts/interval */
	int Run(std::vector<double>& series)
	{
		unsigned ts = this->m_Eng_Interface->GetNumberOfTimesteps();
		bool in = ts >= this->startTS && ts <= this->stopTS;
		int next = this->Process();
		if (in && this->ProcessInterval && ts % this->ProcessInterval == 0) {
			size_t slot = ts / this->ProcessInterval;
			if (slot < series.size())
				series[slot] = this->m_Results[0] * this->m_weight;
		}
		return next;
	}
	void Dft(double* out) const
	{
		for (size_t f = 0; f < this->m_FD_Samples.size(); ++f) {
			out[2 * f] = this->m_FD_Results[0].at(f).real();
			out[2 * f + 1] = this->m_FD_Results[0].at(f).imag();
		}
	}
	size_t NumFreqs() const { return this->m_FD_Samples.size(); }
	unsigned FdInterval() const { return this->m_FD_Interval; }
};

struct ProbeRun {
	ProbeDef def;
	HProbe<ProcessVoltage>* v = nullptr;
	HProbe<ProcessCurrent>* c = nullptr;
	std::vector<double> series;
};

} // namespace

/* ---------------------------------------------------------------------------------------- */
/* engine handle                                                                            */

struct oems_refeng {
	int kind = 0;
	unsigned nthreads = 1;
	unsigned N[3] = {0, 0, 0};
	double dt = 0;
	std::vector<double> lines;
	double unit = 1.0;
	std::string scratch;

	HOp<Operator>* op_basic = nullptr;
	HOp<Operator_sse>* op_sse = nullptr;
	HOpC* op_c = nullptr;
	HOpMT* op_mt = nullptr;
	Operator* op = nullptr;

	HExcitation* exc = nullptr;
	bool exc_built = false; /* signal built by Excitation::buildExcitationSignal */
	bool coeffs = false;
	std::vector<HExtMur*> murs;
	std::vector<HExtUPML*> upmls;
	std::vector<LorOrder> lor;
	std::vector<ProbeRun> probes;

	Engine* eng = nullptr;
	Engine_Interface_FDTD* eif = nullptr;
	unsigned max_ts = 0;
	int next_interval = INT_MAX;
	fenv_t eng_env;
	bool inited = false;
	std::string err;
};

typedef oems_refeng eng_t;

namespace {

/* applies the engine's floating-point state while the engine computes, restores the caller's */
struct FpGuard {
	fenv_t saved;
	eng_t* e;
	explicit FpGuard(eng_t* e_) : e(e_)
	{
		fegetenv(&saved);
		if (e && e->inited)
			fesetenv(&e->eng_env);
	}
	~FpGuard()
	{
		if (e && e->inited)
			fegetenv(&e->eng_env);
		fesetenv(&saved);
	}
};

int fail(eng_t* e, int rc, const std::string& msg)
{
	if (e)
		e->err = msg;
	return rc;
}

void run_probes(eng_t* e)
{
	int next = INT_MAX;
	for (ProbeRun& p : e->probes) {
		int r = p.v ? p.v->Run(p.series) : p.c->Run(p.series);
		if (r > 0 && r < next)
			next = r;
	}
	e->next_interval = next;
}

} // namespace

extern "C" {

/* kind: 0 Engine (basic), 1 Engine_sse, 2 Engine_SSE_Compressed, 3 Engine_Multithread.
 * lines: the mesh lines of x, y, z concatenated in drawing units (NULL: 0,1,2,...), unit in metres.
 * scratch: directory for the probes' text files (the reference writes one per probe). */
int oems_refeng_create_ex(const unsigned nl[3], const double* lines, double unit, double dt, int kind,
                          unsigned nthreads, const char* scratch, eng_t** out)
{
	if (!nl || !out || nl[0] < 2 || nl[1] < 2 || nl[2] < 2 || !(dt > 0) || kind < 0 || kind > 3)
		return ERR_ARG;
	FpGuard g(nullptr);
	eng_t* e = new eng_t();
	e->kind = kind;
	e->nthreads = nthreads ? nthreads : 1;
	for (int n = 0; n < 3; ++n)
		e->N[n] = nl[n];
	e->dt = dt;
	e->unit = unit;
	e->scratch = scratch ? scratch : ".";
	switch (kind) {
	case KIND_BASIC:
		e->op_basic = new HOp<Operator>();
		e->op_basic->SetMesh(nl, lines, unit, dt);
		e->op = e->op_basic;
		break;
	case KIND_SSE:
		e->op_sse = new HOp<Operator_sse>();
		e->op_sse->SetMesh(nl, lines, unit, dt);
		e->op = e->op_sse;
		break;
	case KIND_SSE_COMPRESSED:
		e->op_c = new HOpC();
		e->op_c->SetMesh(nl, lines, unit, dt);
		e->op = e->op_c;
		break;
	default:
		e->op_mt = new HOpMT();
		e->op_mt->SetMesh(nl, lines, unit, dt);
		e->op = e->op_mt;
		break;
	}
	e->exc = new HExcitation();
	e->exc->Reset(dt);
	e->op->SetExcitationSignal(e->exc);
	*out = e;
	return OK;
}

/* the ABI shape of oems_cuda_create: basic engine, mesh lines 0..N-1 */
int oems_refeng_create(const unsigned nl[3], double dt, int device, eng_t** out)
{
	(void)device;
	return oems_refeng_create_ex(nl, nullptr, 1.0, dt, KIND_BASIC, 1, nullptr, out);
}

void oems_refeng_destroy(eng_t* e)
{
	if (!e)
		return;
	FpGuard g(e);
	for (ProbeRun& p : e->probes) {
		delete p.v;
		delete p.c;
	}
	e->probes.clear();
	delete e->eif; /* not owned by the probes: each probe holds its own interface */
	e->eif = nullptr;
	if (e->eng) {
		delete e->eng; /* Engine_Multithread::Reset stops and joins its worker threads */
		e->eng = nullptr;
	}
	if (e->op_basic) e->op_basic->ForgetEngine();
	if (e->op_sse) e->op_sse->ForgetEngine();
	if (e->op_c) e->op_c->ForgetEngine();
	if (e->op_mt) e->op_mt->ForgetEngine();
	delete e->op; /* deletes its extensions */
	e->op = nullptr;
	delete e->exc;
	delete e;
}

const char* oems_refeng_last_error(const eng_t* e)
{
	return e ? e->err.c_str() : "null engine";
}

/* Build the excitation signal with the reference's Excitation (FDTD/excitation.cpp):
 * kind 0 Gaussian (f0, fc), 1 sinusoidal (f0), 2 Dirac (fmax), 3 step (fmax). */
int oems_refeng_set_signal(eng_t* e, int kind, double f0, double fc, double fmax, unsigned max_ts)
{
	if (!e || e->inited)
		return ERR_STATE;
	FpGuard g(e);
	switch (kind) {
	case 0: e->exc->SetupGaussianPulse(f0, fc); break;
	case 1: e->exc->SetupSinusoidal(f0); break;
	case 2: e->exc->SetupDiracPulse(fmax); break;
	case 3: e->exc->SetupStepExcite(fmax); break;
	default: return fail(e, ERR_UNSUPPORTED, "unsupported excitation type");
	}
	e->exc->Reset(e->dt);
	if (!e->exc->buildExcitationSignal(max_ts))
		return fail(e, ERR_ARG, "Excitation::buildExcitationSignal failed");
	e->exc_built = true;
	return OK;
}

/* the signal the reference built: length, nyquist number, period in steps, both arrays (cap floats) */
int oems_refeng_read_signal(eng_t* e, float* v, float* c, unsigned cap, unsigned* len, unsigned* nyquist,
                            unsigned* period)
{
	if (!e || !len)
		return ERR_ARG;
	unsigned L = e->exc->GetLength();
	*len = L;
	if (nyquist)
		*nyquist = e->exc->GetNyquistNum();
	if (period)
		*period = e->exc->GetSignalPeriod() > 0 ? (unsigned)int(e->exc->GetSignalPeriod() / e->exc->GetTimestep()) : 0;
	for (unsigned n = 0; n < L && n < cap; ++n) {
		if (v) v[n] = e->exc->GetVoltageSignal()[n];
		if (c) c[n] = e->exc->GetCurrentSignal()[n];
	}
	return OK;
}

int oems_refeng_set_operator(eng_t* e, const float* vv, const float* vi, const float* ii, const float* iv,
                             unsigned max_classes)
{
	(void)max_classes;
	if (!e || !vv || !vi || !ii || !iv)
		return ERR_ARG;
	if (e->inited)
		return ERR_STATE;
	FpGuard g(e);
	Operator* op = e->op;
	if (e->op_basic) e->op_basic->AllocCoefficients();
	if (e->op_sse) e->op_sse->AllocCoefficients();
	if (e->op_c) e->op_c->AllocCoefficients();
	if (e->op_mt) e->op_mt->AllocCoefficients();
	const unsigned* N = e->N;
	size_t k = 0;
	for (unsigned n = 0; n < 3; ++n)
		for (unsigned x = 0; x < N[0]; ++x)
			for (unsigned y = 0; y < N[1]; ++y)
				for (unsigned z = 0; z < N[2]; ++z, ++k) {
					op->SetVV(n, x, y, z, vv[k]);
					op->SetVI(n, x, y, z, vi[k]);
					op->SetII(n, x, y, z, ii[k]);
					op->SetIV(n, x, y, z, iv[k]);
				}
	if (e->op_c && !e->op_c->Compress())
		return fail(e, ERR_STATE, "CompressOperator failed");
	if (e->op_mt && !e->op_mt->Compress())
		return fail(e, ERR_STATE, "CompressOperator failed");
	e->coeffs = true;
	return OK;
}

int oems_refeng_operator_classes(const eng_t* e, unsigned* nc)
{
	if (!e || !nc)
		return ERR_ARG;
	*nc = e->op_c ? (unsigned)e->op_c->Classes() : e->op_mt ? (unsigned)e->op_mt->Classes() : 0;
	return OK;
}

/* Operator_Ext_Excitation's tables (setupVoltageExcitation / setupCurrentExcitation).  When the
 * signal was built by oems_refeng_set_signal, the given arrays must equal it bit for bit (the
 * call fails otherwise, naming the first difference); else they are used as given. */
int oems_refeng_set_excitation(eng_t* e, unsigned nV, const unsigned* vidx, const unsigned short* vdir,
                               const float* vamp, const unsigned* vdel, unsigned nI, const unsigned* cidx,
                               const unsigned short* cdir, const float* camp, const unsigned* cdel,
                               const float* sig_v, const float* sig_i, unsigned len, unsigned period)
{
	if (!e)
		return ERR_ARG;
	if (e->inited)
		return ERR_STATE;
	FpGuard g(e);
	if (e->exc_built) {
		unsigned L = e->exc->GetLength();
		if (L != len)
			return fail(e, ERR_ARG, "excitation length " + std::to_string(len) + " differs from the reference's " +
			                            std::to_string(L));
		for (unsigned n = 0; n < L; ++n) {
			if (memcmp(&sig_v[n], &e->exc->GetVoltageSignal()[n], 4) != 0 ||
			    memcmp(&sig_i[n], &e->exc->GetCurrentSignal()[n], 4) != 0)
				return fail(e, ERR_ARG, "excitation signal differs from the reference's at index " + std::to_string(n));
		}
		unsigned p = e->exc->GetSignalPeriod() > 0 ? (unsigned)int(e->exc->GetSignalPeriod() / e->exc->GetTimestep()) : 0;
		if (p != period)
			return fail(e, ERR_ARG, "excitation period " + std::to_string(period) + " differs from the reference's " +
			                            std::to_string(p));
	} else {
		e->exc->Inject(sig_v, sig_i, len, period);
	}
	HExtExcitation* x = new HExtExcitation(e->op);
	static const unsigned zero = 0;
	static const unsigned short zs = 0;
	static const float zf = 0;
	x->Fill(e->exc, nV, nV ? vidx : &zero, nV ? vdir : &zs, nV ? vamp : &zf, nV ? vdel : &zero, nI,
	        nI ? cidx : &zero, nI ? cdir : &zs, nI ? camp : &zf, nI ? cdel : &zero);
	/* openems.cpp:1186: the excitation extension is added first */
	e->op->AddExtension(x);
	return OK;
}

int oems_refeng_add_upml(eng_t* e, const unsigned start[3], const unsigned nl[3], const float* vv, const float* vvfo,
                         const float* vvfn, const float* ii, const float* iifo, const float* iifn)
{
	if (!e || !start || !nl)
		return ERR_ARG;
	if (e->inited)
		return ERR_STATE;
	FpGuard g(e);
	HExtUPML* u = new HExtUPML(e->op);
	const float* tab[6] = {vv, vvfo, vvfn, ii, iifo, iifn};
	u->Fill(start, nl, tab);
	e->upmls.push_back(u);
	return OK;
}

int oems_refeng_add_mur(eng_t* e, int ny, unsigned line_nr, unsigned line_nr_shift, unsigned start_ts,
                        const float* cP, const float* cPP)
{
	if (!e || ny < 0 || ny > 2 || !cP || !cPP)
		return ERR_ARG;
	if (e->inited)
		return ERR_STATE;
	FpGuard g(e);
	HExtMur* m = new HExtMur(e->op);
	if (!m->Fill(ny, line_nr, cP, cPP) || (unsigned)m->LineShift() != line_nr_shift) {
		delete m;
		return fail(e, ERR_ARG, "Mur wall line does not match SetDirection");
	}
	(void)start_ts; /* the engine extension derives m_start_TS itself (engine_ext_mur_abc.cpp:42-60) */
	e->murs.push_back(m);
	return OK;
}

int oems_refeng_add_lorentz_order(eng_t* e, unsigned count, const unsigned* pos, int von, int con, int vlon,
                                  int clon, const float* v_int, const float* v_ext, const float* v_lor,
                                  const float* i_int, const float* i_ext, const float* i_lor)
{
	if (!e || (count && !pos))
		return ERR_ARG;
	if (e->inited)
		return ERR_STATE;
	LorOrder L;
	L.pos.assign(pos, pos + 3 * (size_t)count);
	L.von = von != 0;
	L.con = con != 0;
	L.vlon = vlon != 0;
	L.clon = clon != 0;
	const float* src[6] = {v_int, v_ext, v_lor, i_int, i_ext, i_lor};
	bool on[6] = {L.von, L.von, L.vlon, L.con, L.con, L.clon};
	for (int a = 0; a < 6; ++a)
		if (on[a]) {
			if (!src[a])
				return ERR_ARG;
			L.t[a].assign(src[a], src[a] + 3 * (size_t)count);
		}
	e->lor.push_back(L);
	return OK;
}

/* features the harness does not drive: the entry points exist so that one driver serves every
 * engine library, and each reports OEMS_ERR_UNSUPPORTED */
int oems_refeng_set_tfsf(eng_t* e, unsigned, const unsigned*, const unsigned short*, const unsigned*, const float*,
                         const float*, unsigned, const unsigned*, const unsigned short*, const unsigned*, const float*,
                         const float*, const float*, const float*, unsigned, unsigned, unsigned)
{
	return fail(e, ERR_UNSUPPORTED, "TFSF is not driven by the harness");
}
int oems_refeng_set_lumped_rlc(eng_t* e, unsigned, const unsigned*, const int*, const float*, const float*, const float*,
                               const float*, const float*, const float*, const float*, const float*, const float*)
{
	return fail(e, ERR_UNSUPPORTED, "lumped RLC is not driven by the harness");
}
int oems_refeng_add_field_probe(eng_t* e, int, const unsigned*, const double*, double, unsigned, unsigned, unsigned, int*)
{
	return fail(e, ERR_UNSUPPORTED, "field probes are not driven by the harness");
}
int oems_refeng_set_cylinder(eng_t* e, int, int, const float*, const float*)
{
	return fail(e, ERR_UNSUPPORTED, "cylindrical meshes are not driven by the harness");
}
int oems_refeng_set_dump_rho(eng_t* e, int, const double*)
{
	return fail(e, ERR_UNSUPPORTED, "field dumps are not driven by the harness");
}
int oems_refeng_add_fd_dump(eng_t* e, int, int, const unsigned*, const unsigned*, unsigned, unsigned, const double*,
                            const double*, const double*, int*)
{
	return fail(e, ERR_UNSUPPORTED, "field dumps are not driven by the harness");
}
int oems_refeng_add_td_dump(eng_t* e, int, int, const unsigned*, const unsigned*, unsigned, unsigned, unsigned,
                            const double*, const double*, const double*, const char*, int*)
{
	return fail(e, ERR_UNSUPPORTED, "field dumps are not driven by the harness");
}
int oems_refeng_read_fd_dump(eng_t* e, int, float*, size_t)
{
	return fail(e, ERR_UNSUPPORTED, "field dumps are not driven by the harness");
}

static int add_probe(eng_t* e, int type, const unsigned* s, const unsigned* t, int norm_dir, const int* si, const int* ei,
                     double weight, unsigned interval, unsigned start_ts, unsigned stop_ts, int* id)
{
	if (!e || !s || !t || !id || interval == 0)
		return ERR_ARG;
	if (e->inited)
		return ERR_STATE;
	ProbeRun p;
	p.def.type = type;
	for (int n = 0; n < 3; ++n) {
		p.def.start[n] = s[n];
		p.def.stop[n] = t[n];
		p.def.si[n] = si ? si[n] : 1;
		p.def.ei[n] = ei ? ei[n] : 1;
	}
	p.def.norm_dir = norm_dir;
	p.def.weight = weight;
	p.def.interval = interval;
	p.def.start_ts = start_ts;
	p.def.stop_ts = stop_ts;
	p.def.fd_interval = 0;
	*id = (int)e->probes.size();
	e->probes.push_back(p);
	return OK;
}

int oems_refeng_add_voltage_probe(eng_t* e, const unsigned* s, const unsigned* t, double weight, unsigned interval,
                                  unsigned start_ts, unsigned stop_ts, int* id)
{
	return add_probe(e, 0, s, t, -1, nullptr, nullptr, weight, interval, start_ts, stop_ts, id);
}

int oems_refeng_add_current_probe(eng_t* e, const unsigned* s, const unsigned* t, int norm_dir, const int* si,
                                  const int* ei, double weight, unsigned interval, unsigned start_ts, unsigned stop_ts,
                                  int* id)
{
	return add_probe(e, 1, s, t, norm_dir, si, ei, weight, interval, start_ts, stop_ts, id);
}

int oems_refeng_set_probe_dft(eng_t* e, int id, unsigned fd_interval, unsigned nf, const double* freqs)
{
	if (!e || id < 0 || id >= (int)e->probes.size() || (nf && !freqs))
		return ERR_ARG;
	if (e->inited)
		return ERR_STATE;
	e->probes[id].def.fd_interval = fd_interval;
	e->probes[id].def.freqs.assign(freqs, freqs + nf);
	return OK;
}

int oems_refeng_init(eng_t* e, unsigned max_ts)
{
	if (!e || e->inited)
		return ERR_STATE;
	if (!e->coeffs)
		return fail(e, ERR_STATE, "operator not set");
	FpGuard g(e);
	/* openems.cpp:1186-1241 and 383-407: excitation (already added), Mur walls, UPML, Lorentz */
	for (HExtMur* m : e->murs)
		e->op->AddExtension(m);
	for (HExtUPML* u : e->upmls)
		e->op->AddExtension(u);
	if (!e->lor.empty()) {
		HExtLorentz* l = new HExtLorentz(e->op);
		l->Fill(e->lor);
		e->op->AddExtension(l);
	}
	bool has_exc = false;
	for (size_t n = 0; n < e->op->GetNumberOfExtentions(); ++n)
		if (dynamic_cast<Operator_Ext_Excitation*>(e->op->GetExtension(n)))
			has_exc = true;
	if (!has_exc)
		return fail(e, ERR_STATE, "excitation not set");

	/* Operator::CreateEngine of each operator type (the multithreaded one with a fixed thread count) */
	switch (e->kind) {
	case KIND_BASIC:
		e->eng = Engine::New(e->op_basic);
		e->op_basic->SetEngine(e->eng);
		break;
	case KIND_SSE:
		e->eng = Engine_sse::New(e->op_sse);
		e->op_sse->SetEngine(e->eng);
		break;
	case KIND_SSE_COMPRESSED:
		e->eng = Engine_SSE_Compressed::New(e->op_c);
		e->op_c->SetEngine(e->eng);
		break;
	default:
		e->eng = Engine_Multithread::New(e->op_mt, e->nthreads);
		e->op_mt->SetEngine(e->eng);
		break;
	}
	/* the engine's floating-point state from here on (FTZ/DAZ where the engine set it) */
	fegetenv(&e->eng_env);
	e->inited = true;
	e->max_ts = max_ts;
	e->eif = new Engine_Interface_FDTD(e->op);
	for (size_t k = 0; k < e->probes.size(); ++k) {
		ProbeRun& p = e->probes[k];
		p.series.assign(max_ts / p.def.interval + 1, std::numeric_limits<double>::quiet_NaN());
		std::string name = e->scratch + "/refeng_probe_" + std::to_string((unsigned long)(uintptr_t)e) + "_" +
		                   std::to_string(k);
		unsigned fdi;
		if (p.def.type == 0) {
			p.v = new HProbe<ProcessVoltage>(new Engine_Interface_FDTD(e->op), p.def, name);
			fdi = p.v->FdInterval();
		} else {
			p.c = new HProbe<ProcessCurrent>(new Engine_Interface_FDTD(e->op), p.def, name);
			fdi = p.c->FdInterval();
		}
		if (!p.def.freqs.empty() && p.def.fd_interval && fdi != p.def.fd_interval)
			return fail(e, ERR_ARG, "probe " + std::to_string(k) + ": DFT interval " + std::to_string(p.def.fd_interval) +
			                            " differs from the reference's " + std::to_string(fdi));
	}
	/* openEMS::RunFDTD processes once before the first step */
	run_probes(e);
	return OK;
}

int oems_refeng_iterate(eng_t* e, unsigned n)
{
	if (!e || !e->inited)
		return ERR_STATE;
	FpGuard g(e);
	unsigned left = n;
	while (left) {
		unsigned chunk = left;
		if (!e->probes.empty() && e->next_interval > 0 && (unsigned)e->next_interval < chunk)
			chunk = (unsigned)e->next_interval;
		e->eng->IterateTS(chunk);
		left -= chunk;
		if (!e->probes.empty())
			run_probes(e);
	}
	return OK;
}

int oems_refeng_sync(eng_t* e) { return e ? OK : ERR_ARG; }

unsigned oems_refeng_num_timesteps(const eng_t* e)
{
	return e && e->eng ? e->eng->GetNumberOfTimesteps() : 0;
}

int oems_refeng_read_field(eng_t* e, int which, float* out)
{
	if (!e || !out || (which != 0 && which != 1))
		return ERR_ARG;
	if (!e->inited)
		return ERR_STATE;
	FpGuard g(e);
	size_t k = 0;
	for (unsigned n = 0; n < 3; ++n)
		for (unsigned x = 0; x < e->N[0]; ++x)
			for (unsigned y = 0; y < e->N[1]; ++y)
				for (unsigned z = 0; z < e->N[2]; ++z, ++k)
					out[k] = which ? e->eng->GetCurr(n, x, y, z) : e->eng->GetVolt(n, x, y, z);
	return OK;
}

int oems_refeng_write_field(eng_t* e, int which, const float* in)
{
	if (!e || !in || (which != 0 && which != 1))
		return ERR_ARG;
	if (!e->inited)
		return ERR_STATE;
	FpGuard g(e);
	size_t k = 0;
	for (unsigned n = 0; n < 3; ++n)
		for (unsigned x = 0; x < e->N[0]; ++x)
			for (unsigned y = 0; y < e->N[1]; ++y)
				for (unsigned z = 0; z < e->N[2]; ++z, ++k) {
					if (which)
						e->eng->SetCurr(n, x, y, z, in[k]);
					else
						e->eng->SetVolt(n, x, y, z, in[k]);
				}
	return OK;
}

int oems_refeng_get_value(eng_t* e, int which, unsigned n, unsigned x, unsigned y, unsigned z, float* v)
{
	if (!e || !v || n > 2 || x >= e->N[0] || y >= e->N[1] || z >= e->N[2])
		return ERR_ARG;
	if (!e->inited)
		return ERR_STATE;
	*v = which ? e->eng->GetCurr(n, x, y, z) : e->eng->GetVolt(n, x, y, z);
	return OK;
}

int oems_refeng_set_value(eng_t* e, int which, unsigned n, unsigned x, unsigned y, unsigned z, float v)
{
	if (!e || n > 2 || x >= e->N[0] || y >= e->N[1] || z >= e->N[2])
		return ERR_ARG;
	if (!e->inited)
		return ERR_STATE;
	if (which)
		e->eng->SetCurr(n, x, y, z, v);
	else
		e->eng->SetVolt(n, x, y, z, v);
	return OK;
}

int oems_refeng_read_probe(eng_t* e, int id, double* out, size_t cap, size_t* count)
{
	if (!e || id < 0 || id >= (int)e->probes.size() || !out || !count)
		return ERR_ARG;
	const std::vector<double>& s = e->probes[id].series;
	size_t n = s.size() < cap ? s.size() : cap;
	memcpy(out, s.data(), n * sizeof(double));
	*count = n;
	return OK;
}

int oems_refeng_read_probe_dft(eng_t* e, int id, double* out)
{
	if (!e || id < 0 || id >= (int)e->probes.size() || !out)
		return ERR_ARG;
	if (!e->inited)
		return ERR_STATE;
	ProbeRun& p = e->probes[id];
	if (p.v)
		p.v->Dft(out);
	else
		p.c->Dft(out);
	return OK;
}

int oems_refeng_energy(eng_t* e, double* out)
{
	if (!e || !out)
		return ERR_ARG;
	if (!e->inited)
		return ERR_STATE;
	FpGuard g(e);
	*out = e->eif->CalcFastEnergy();
	return OK;
}

/* x-slab split of the multithreaded engine (Operator_Multithread::CalcStartStopLines) */
int oems_refeng_thread_lines(eng_t* e, unsigned* nthreads, unsigned* start, unsigned* stop, unsigned cap)
{
	if (!e || !nthreads || !e->op_mt)
		return ERR_ARG;
	std::vector<unsigned int> a, b;
	unsigned t = e->nthreads;
	e->op_mt->ThreadLines(t, a, b);
	*nthreads = t;
	for (unsigned k = 0; k < t && k < cap; ++k) {
		if (start) start[k] = a[k];
		if (stop) stop[k] = b[k];
	}
	return OK;
}

} /* extern "C" */
