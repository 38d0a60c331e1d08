/*
 * engine_cuda.cpp -- the openEMS-side binding of the GB300 engine; see engine_cuda.h.
 */
#include "engine_cuda.h"

#include <algorithm>
#include <cmath>

#include "FDTD/excitation.h"
#include "FDTD/extensions/operator_ext_excitation.h"
#include "FDTD/extensions/operator_ext_lorentzmaterial.h"
#include "FDTD/extensions/operator_ext_mur_abc.h"
#include "FDTD/extensions/operator_ext_upml.h"

namespace {

// Read access to the protected tables of the operator extensions: a member pointer formed inside
// a derived class has the base class's member type and applies to any object of the base.
struct ExcAccess : Operator_Ext_Excitation {
	static constexpr auto VoltCount = &ExcAccess::Volt_Count;
	static constexpr auto VoltIndex = &ExcAccess::Volt_index;
	static constexpr auto VoltDir = &ExcAccess::Volt_dir;
	static constexpr auto VoltAmp = &ExcAccess::Volt_amp;
	static constexpr auto VoltDelay = &ExcAccess::Volt_delay;
	static constexpr auto CurrCount = &ExcAccess::Curr_Count;
	static constexpr auto CurrIndex = &ExcAccess::Curr_index;
	static constexpr auto CurrDir = &ExcAccess::Curr_dir;
	static constexpr auto CurrAmp = &ExcAccess::Curr_amp;
	static constexpr auto CurrDelay = &ExcAccess::Curr_delay;
};
struct UpmlAccess : Operator_Ext_UPML {
	static constexpr auto StartPos = &UpmlAccess::m_StartPos;
	static constexpr auto NumLines = &UpmlAccess::m_numLines;
	static constexpr auto VV = &UpmlAccess::vv;
	static constexpr auto VVFO = &UpmlAccess::vvfo;
	static constexpr auto VVFN = &UpmlAccess::vvfn;
	static constexpr auto II = &UpmlAccess::ii;
	static constexpr auto IIFO = &UpmlAccess::iifo;
	static constexpr auto IIFN = &UpmlAccess::iifn;
};
struct MurAccess : Operator_Ext_Mur_ABC {
	static constexpr auto Ny = &MurAccess::m_ny;
	static constexpr auto NyP = &MurAccess::m_nyP;
	static constexpr auto NyPP = &MurAccess::m_nyPP;
	static constexpr auto LineNr = &MurAccess::m_LineNr;
	static constexpr auto LineShift = &MurAccess::m_LineNr_Shift;
	static constexpr auto CoeffP = &MurAccess::m_Mur_Coeff_nyP;
	static constexpr auto CoeffPP = &MurAccess::m_Mur_Coeff_nyPP;
};
struct LorAccess : Operator_Ext_LorentzMaterial {
	static constexpr auto Order = &LorAccess::m_Order;
	static constexpr auto Count = &LorAccess::m_LM_Count;
	static constexpr auto Pos = &LorAccess::m_LM_pos;
	static constexpr auto VoltOn = &LorAccess::m_volt_ADE_On;
	static constexpr auto CurrOn = &LorAccess::m_curr_ADE_On;
	static constexpr auto VoltLorOn = &LorAccess::m_volt_Lor_ADE_On;
	static constexpr auto CurrLorOn = &LorAccess::m_curr_Lor_ADE_On;
	static constexpr auto VInt = &LorAccess::v_int_ADE;
	static constexpr auto VExt = &LorAccess::v_ext_ADE;
	static constexpr auto VLor = &LorAccess::v_Lor_ADE;
	static constexpr auto IInt = &LorAccess::i_int_ADE;
	static constexpr auto IExt = &LorAccess::i_ext_ADE;
	static constexpr auto ILor = &LorAccess::i_Lor_ADE;
};
struct SSECAccess : Operator_SSE_Compressed {
	static constexpr auto NumVectors = &SSECAccess::numVectors;
};

std::vector<unsigned> flat3(unsigned* const idx[3], unsigned count)
{
	std::vector<unsigned> out(3 * (size_t)count);
	for (int n = 0; n < 3; ++n)
		std::copy(idx[n], idx[n] + count, out.begin() + (size_t)n * count);
	return out;
}

// steps per signal period, as Engine_Ext_Excitation derives p (engine_ext_excitation.cpp:41-43)
unsigned period_steps(const Excitation* exc)
{
	if (exc->GetSignalPeriod() > 0)
		return (unsigned)int(exc->GetSignalPeriod() / exc->GetTimestep());
	return 0;
}

} // namespace

Operator_CUDA* Operator_CUDA::New()
{
	Operator_CUDA* op = new Operator_CUDA();
	op->Init();
	return op;
}

Engine* Operator_CUDA::CreateEngine()
{
	// the device engine reads the compressed tables; they exist after CalcECOperator
	if (!m_Use_Compression)
		throw std::runtime_error("engine cuda: the operator was not compressed");
	m_Engine = Engine_CUDA::New(this);
	return m_Engine;
}

Engine_CUDA* Engine_CUDA::New(const Operator_CUDA* op, int device)
{
	Engine_CUDA* e = new Engine_CUDA(op, device);
	e->Init();
	return e;
}

Engine_CUDA::Engine_CUDA(const Operator_CUDA* op, int device)
	: Engine(op), m_OpCUDA(op), m_device(device), m_h(nullptr), m_started(false)
{
	m_type = UNKNOWN;
}

Engine_CUDA::~Engine_CUDA()
{
	Reset();
}

void Engine_CUDA::Check(int rc, const char* what) const
{
	if (rc != OEMS_OK)
		throw std::runtime_error(std::string("engine cuda: ") + what + " failed (" + std::to_string(rc) + "): " +
		                         (m_h ? oems_cuda_last_error(m_h) : ""));
}

void Engine_CUDA::Reset()
{
	if (m_h)
		oems_cuda_destroy(m_h);
	m_h = nullptr;
	m_started = false;
	Engine::Reset();
}

void Engine_CUDA::Init()
{
	numTS = 0;   // no host field arrays: Engine::Init is not called
	unsigned nl[3] = {numLines[0], numLines[1], numLines[2]};
	Check(oems_cuda_create(nl, Op->GetTimestep(), m_device, &m_h), "oems_cuda_create");

	// the reference's own compressed operator (operator_sse_compressed.h:70-85), lane-strided z
	const Operator_SSE_Compressed* sc = m_OpCUDA;
	const unsigned U = (unsigned)sc->f4_vv_Compressed[0].size();
	std::vector<float> t[4];
	const std::vector<f4vector, aligned_allocator<f4vector>>* src[4] = {sc->f4_vv_Compressed, sc->f4_vi_Compressed,
	                                                                     sc->f4_ii_Compressed, sc->f4_iv_Compressed};
	for (int a = 0; a < 4; ++a) {
		t[a].resize(3 * (size_t)U * 4);
		for (int n = 0; n < 3; ++n)
			for (unsigned u = 0; u < U; ++u)
				for (int l = 0; l < 4; ++l)
					t[a][((size_t)n * U + u) * 4 + l] = src[a][n][u].f[l];
	}
	const unsigned nv = sc->*SSECAccess::NumVectors;
	std::vector<unsigned> index((size_t)nl[0] * nl[1] * nv);
	for (unsigned x = 0; x < nl[0]; ++x)
		for (unsigned y = 0; y < nl[1]; ++y)
			for (unsigned v = 0; v < nv; ++v)
				index[((size_t)x * nl[1] + y) * nv + v] = sc->m_Op_index(x, y, v);
	Check(oems_cuda_set_operator_sse_compressed(m_h, U, t[0].data(), t[1].data(), t[2].data(), t[3].data(),
	                                            index.data()),
	      "oems_cuda_set_operator_sse_compressed");

	// the extensions, in the operator's order (the device engine applies the reference's
	// priority order itself)
	Operator_Ext_Excitation* exc = Op->GetExcitationExtension();
	for (size_t k = 0; k < Op->GetNumberOfExtentions(); ++k) {
		Operator_Extension* x = Op->GetExtension(k);
		if (auto* ex = dynamic_cast<Operator_Ext_Excitation*>(x)) {
			const Excitation* sig = Op->GetExcitationSignal();
			const unsigned nV = ex->*ExcAccess::VoltCount, nI = ex->*ExcAccess::CurrCount;
			std::vector<unsigned> vi = flat3(ex->*ExcAccess::VoltIndex, nV), ci = flat3(ex->*ExcAccess::CurrIndex, nI);
			Check(oems_cuda_set_excitation(m_h, nV, vi.data(), ex->*ExcAccess::VoltDir, ex->*ExcAccess::VoltAmp,
			                               ex->*ExcAccess::VoltDelay, nI, ci.data(), ex->*ExcAccess::CurrDir,
			                               ex->*ExcAccess::CurrAmp, ex->*ExcAccess::CurrDelay, sig->GetVoltageSignal(),
			                               sig->GetCurrentSignal(), sig->GetLength(), period_steps(sig)),
			      "oems_cuda_set_excitation");
		} else if (auto* u = dynamic_cast<Operator_Ext_UPML*>(x)) {
			Check(oems_cuda_add_upml(m_h, u->*UpmlAccess::StartPos, u->*UpmlAccess::NumLines, (u->*UpmlAccess::VV).data(),
			                         (u->*UpmlAccess::VVFO).data(), (u->*UpmlAccess::VVFN).data(),
			                         (u->*UpmlAccess::II).data(), (u->*UpmlAccess::IIFO).data(),
			                         (u->*UpmlAccess::IIFN).data()),
			      "oems_cuda_add_upml");
		} else if (auto* m = dynamic_cast<Operator_Ext_Mur_ABC*>(x)) {
			// m_start_TS as Engine_Ext_Mur_ABC derives it (engine_ext_mur_abc.cpp:42-60)
			const int ny = m->*MurAccess::Ny, nyP = m->*MurAccess::NyP, nyPP = m->*MurAccess::NyPP;
			const unsigned line = m->*MurAccess::LineNr;
			int maxDelay = -1;
			if (exc) {
				const unsigned nV = exc->*ExcAccess::VoltCount;
				unsigned* const* vidx = exc->*ExcAccess::VoltIndex;
				for (unsigned n = 0; n < nV; ++n) {
					const unsigned short d = (exc->*ExcAccess::VoltDir)[n];
					if ((d == nyP || d == nyPP) && vidx[ny][n] == line)
						maxDelay = std::max(maxDelay, (int)(exc->*ExcAccess::VoltDelay)[n]);
				}
			}
			const unsigned start_ts = maxDelay >= 0 ? maxDelay + Op->GetExcitationSignal()->GetLength() + 10 : 0;
			Check(oems_cuda_add_mur(m_h, ny, line, (unsigned)(m->*MurAccess::LineShift), start_ts,
			                        (m->*MurAccess::CoeffP).data(), (m->*MurAccess::CoeffPP).data()),
			      "oems_cuda_add_mur");
		} else if (auto* l = dynamic_cast<Operator_Ext_LorentzMaterial*>(x)) {
			const int order = l->*LorAccess::Order;
			for (int o = 0; o < order; ++o) {
				const unsigned M = (l->*LorAccess::Count)[o];
				std::vector<unsigned> pos = flat3((l->*LorAccess::Pos)[o], M);
				const bool von = (l->*LorAccess::VoltOn)[o], con = (l->*LorAccess::CurrOn)[o];
				const bool vlon = (l->*LorAccess::VoltLorOn)[o], clon = (l->*LorAccess::CurrLorOn)[o];
				auto tab = [&](FDTD_FLOAT*** a, bool on) {
					std::vector<float> out;
					if (on)
						for (int n = 0; n < 3; ++n)
							out.insert(out.end(), a[o][n], a[o][n] + M);
					return out;
				};
				std::vector<float> vint = tab(l->*LorAccess::VInt, von), vext = tab(l->*LorAccess::VExt, von);
				std::vector<float> vlor = tab(l->*LorAccess::VLor, vlon), iint = tab(l->*LorAccess::IInt, con);
				std::vector<float> iext = tab(l->*LorAccess::IExt, con), ilor = tab(l->*LorAccess::ILor, clon);
				auto ptr = [](std::vector<float>& v) { return v.empty() ? nullptr : v.data(); };
				Check(oems_cuda_add_lorentz_order(m_h, M, pos.data(), von, con, vlon, clon, ptr(vint), ptr(vext),
				                                  ptr(vlor), ptr(iint), ptr(iext), ptr(ilor)),
				      "oems_cuda_add_lorentz_order");
			}
		} else {
			// TFSF, lumped RLC and the cylinder extension have entry points of their own
			// (oems_cuda_set_tfsf, _set_lumped_rlc, _set_cylinder); this binding hands over the
			// extensions of the engine's core path
			throw std::runtime_error("engine cuda: extension not handed over by this binding: " + x->GetExtensionName());
		}
	}
}

void Engine_CUDA::StartRun(unsigned int maxTS)
{
	Check(oems_cuda_init(m_h, maxTS), "oems_cuda_init");
	m_started = true;
}

bool Engine_CUDA::IterateTS(unsigned int iterTS)
{
	if (!m_started)
		StartRun(iterTS);
	Check(oems_cuda_iterate(m_h, iterTS), "oems_cuda_iterate");
	numTS = oems_cuda_num_timesteps(m_h);
	return true;
}

unsigned int Engine_CUDA::GetNumberOfTimesteps()
{
	return m_h ? oems_cuda_num_timesteps(m_h) : numTS;
}

FDTD_FLOAT Engine_CUDA::GetVolt(unsigned int n, unsigned int x, unsigned int y, unsigned int z) const
{
	float v = 0;
	Check(oems_cuda_get_value(m_h, OEMS_VOLT, n, x, y, z, &v), "oems_cuda_get_value");
	return v;
}

FDTD_FLOAT Engine_CUDA::GetVolt(unsigned int n, const unsigned int pos[3]) const
{
	return GetVolt(n, pos[0], pos[1], pos[2]);
}

FDTD_FLOAT Engine_CUDA::GetCurr(unsigned int n, unsigned int x, unsigned int y, unsigned int z) const
{
	float v = 0;
	Check(oems_cuda_get_value(m_h, OEMS_CURR, n, x, y, z, &v), "oems_cuda_get_value");
	return v;
}

FDTD_FLOAT Engine_CUDA::GetCurr(unsigned int n, const unsigned int pos[3]) const
{
	return GetCurr(n, pos[0], pos[1], pos[2]);
}

void Engine_CUDA::SetVolt(unsigned int n, unsigned int x, unsigned int y, unsigned int z, FDTD_FLOAT value)
{
	Check(oems_cuda_set_value(m_h, OEMS_VOLT, n, x, y, z, value), "oems_cuda_set_value");
}

void Engine_CUDA::SetVolt(unsigned int n, const unsigned int pos[3], FDTD_FLOAT value)
{
	SetVolt(n, pos[0], pos[1], pos[2], value);
}

void Engine_CUDA::SetCurr(unsigned int n, unsigned int x, unsigned int y, unsigned int z, FDTD_FLOAT value)
{
	Check(oems_cuda_set_value(m_h, OEMS_CURR, n, x, y, z, value), "oems_cuda_set_value");
}

void Engine_CUDA::SetCurr(unsigned int n, const unsigned int pos[3], FDTD_FLOAT value)
{
	SetCurr(n, pos[0], pos[1], pos[2], value);
}
