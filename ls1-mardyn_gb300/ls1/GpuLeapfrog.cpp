/*
 * GpuLeapfrog.cpp -- see GpuLeapfrog.h.
 */
#include "GpuLeapfrog.h"

#include <sstream>

#include "Domain.h"
#include "GpuLinkedCells.h"
#include "utils/Logger.h"
#include "utils/mardyn_assert.h"
#include "utils/xmlfileUnits.h"

namespace {
GpuLinkedCells* gpuContainer(ParticleContainer* c) {
	auto* g = dynamic_cast<GpuLinkedCells*>(c);
	if (!g) MARDYN_EXIT("GpuLeapfrog needs <datastructure type=\"GpuLinkedCells\">");
	return g;
}

void check(md_ctx* ctx, int rc, const char* what) {
	if (rc != MD_OK) {
		std::ostringstream msg;
		msg << "GpuLeapfrog: " << what << " failed (" << rc << "): " << md_last_error(ctx) << std::endl;
		MARDYN_EXIT(msg.str());
	}
}
}  // namespace

void GpuLeapfrog::readXML(XMLfileUnits& xmlconfig) {
	_timestepLength = 0;
	xmlconfig.getNodeValueReduced("timestep", _timestepLength);
	Log::global_log->info() << "GpuLeapfrog timestep: " << _timestepLength << std::endl;
}

void GpuLeapfrog::eventNewTimestep(ParticleContainer* moleculeContainer, Domain* /*domain*/) {
	GpuLinkedCells* g = gpuContainer(moleculeContainer);
	md_ctx* ctx = g->deviceContext();
	check(ctx, md_integrate_pre(ctx, _timestepLength), "md_integrate_pre");
	g->deviceStepped();
	_postForcePending = true;
}

void GpuLeapfrog::eventForcesCalculated(ParticleContainer* moleculeContainer, Domain* domain) {
	if (!_postForcePending) return;  // Leapfrog::eventForcesCalculated acts in STATE_PRE_FORCE_CALCULATION only
	GpuLinkedCells* g = gpuContainer(moleculeContainer);
	md_ctx* ctx = g->deviceContext();
	md_kinetic_out k{};
	check(ctx, md_integrate_post(ctx, _timestepLength, &k), "md_integrate_post");
	g->deviceStepped();
	domain->setLocalSummv2(k.summv2, 0);
	domain->setLocalSumIw2(k.sumIw2, 0);
	domain->setLocalNrotDOF(0, (unsigned long)k.n, (unsigned long)k.rot_dof);
	_postForcePending = false;
}
