// Test-infrastructure driver around the reference implementation's reduced
// memory mode (built with -DENABLE_REDUCED_MEMORY_MODE by the Makefile beside
// it, RMM=1).  It is linked against the reference's objects and only prints
// what the reference computes; it implements no physics of its own.
//
// Mode (all values printed with 17 significant digits):
//   rmmsteps <file.inp> <rc> <rcLJ> <dt> <nsteps>
//       NVE steps of single-centre LJ molecules in the order of the
//       reference's Simulation with the reduced memory mode:
//       prepare_start (Simulation.cpp:895-935): periodic halo, the first
//       traversal with VCP1CLJRMM at half the velocity kick dt/(2m);
//       simulateOneTimestep: LeapfrogRMM::computePositions
//       (PositionCellProcessorRMM), update + periodic exchange, traversal
//       with VCP1CLJRMM (forces kick the velocities by dt/m inside the pair
//       loop), LeapfrogRMM::computeVelocities (VelocityCellProcessorRMM:
//       N and sum m v^2).  Thermostat off, no long-range correction.
//
// Output records:
//   STEP <k> <Upot> <virial> <summv2>
//   N <count>
//   MOL <id> r[3] v[3]

#include <cstdio>
#include <iostream>
#include <memory>
#include <string>
#include <vector>
#include <algorithm>

#include "Simulation.h"
#include "Domain.h"
#include "ensemble/EnsembleBase.h"
#include "integrators/PositionCellProcessorRMM.h"
#include "integrators/VelocityCellProcessorRMM.h"
#include "io/ASCIIReader.h"
#include "molecules/Molecule.h"
#include "parallel/DomainDecompBase.h"
#include "particleContainer/LinkedCells.h"
#include "particleContainer/adapter/VCP1CLJRMM.h"
#include "particleContainer/adapter/vectorization/SIMD_TYPES.h"
#include "utils/Logger.h"

static_assert(VCP_VEC_TYPE == VCP_NOVEC, "golden vectors come from the scalar kernel path");

namespace {

int runRmmSteps(const std::string& file, double rc, double rcLJ, double dt, int nsteps) {
	new Simulation();  // assigns global_simulation
	Domain* domain = global_simulation->getDomain();
	DomainDecompBase* dd = &global_simulation->domainDecomposition();
	global_simulation->setcutoffRadius(rc);
	global_simulation->setLJCutoff(rcLJ);
	ASCIIReader reader;
	reader.setPhaseSpaceHeaderFile(file);
	reader.setPhaseSpaceFile(file);
	reader.readPhaseSpaceHeader(domain, 1.0);
	double bmin[3], bmax[3];
	for (int d = 0; d < 3; ++d) {
		bmin[d] = dd->getBoundingBoxMin(d, domain);
		bmax[d] = dd->getBoundingBoxMax(d, domain);
	}
	LinkedCells* lc = new LinkedCells(bmin, bmax, rc);
	reader.readPhaseSpace(lc, domain, dd);
	lc->deleteOuterParticles();
	lc->update();
	domain->thermostatOff();

	dd->exchangeMolecules(lc, domain);
	lc->updateMoleculeCaches();
	domain->initParameterStreams(rc, rcLJ);
	VCP1CLJRMM vcp(*domain, rc, rcLJ);
	const double m = global_simulation->getEnsemble()->getComponents()->front().m();
	const double dtInvm = dt / m;
	PositionCellProcessorRMM positions(dt);
	VelocityCellProcessorRMM velocities;

	// initial forces with half the kick (Simulation::prepare_start)
	vcp.setDtInvm(dtInvm * 0.5);
	lc->traverseCells(vcp);
	lc->deleteOuterParticles();
	vcp.setDtInvm(dtInvm);
	std::printf("STEP 0 %.17g %.17g nan\n", domain->getLocalUpot(), domain->getLocalVirial());

	for (int k = 1; k <= nsteps; ++k) {
		lc->traverseCells(positions);  // LeapfrogRMM::eventNewTimestep
		lc->update();
		dd->exchangeMolecules(lc, domain);
		lc->updateMoleculeCaches();
		lc->traverseCells(vcp);
		lc->deleteOuterParticles();
		const double upot = domain->getLocalUpot();
		const double vir = domain->getLocalVirial();
		lc->traverseCells(velocities);  // LeapfrogRMM::eventForcesCalculated
		std::printf("STEP %d %.17g %.17g %.17g\n", k, upot, vir, velocities.getSummv2());
	}

	struct Row { unsigned long id; double v[6]; };
	std::vector<Row> rows;
	for (auto it = lc->iterator(ParticleIterator::ONLY_INNER_AND_BOUNDARY); it.isValid(); ++it) {
		Row r;
		r.id = it->getID();
		for (int d = 0; d < 3; ++d) {
			r.v[d] = it->r(d);
			r.v[3 + d] = it->v(d);
		}
		rows.push_back(r);
	}
	std::sort(rows.begin(), rows.end(), [](const Row& a, const Row& b) { return a.id < b.id; });
	std::printf("N %zu\n", rows.size());
	for (const Row& r : rows) {
		std::printf("MOL %lu", r.id);
		for (double x : r.v) std::printf(" %.17g", x);
		std::printf("\n");
	}
	return 0;
}

}  // namespace

int main(int argc, char** argv) {
	Log::global_log = std::make_unique<Log::Logger>(Log::Warning, std::shared_ptr<std::ostream>(&std::cerr, [](void*) {}));
	if (argc >= 7 && std::string(argv[1]) == "rmmsteps")
		return runRmmSteps(argv[2], std::stod(argv[3]), std::stod(argv[4]), std::stod(argv[5]), std::stoi(argv[6]));
	std::fprintf(stderr, "usage: %s rmmsteps <inp> <rc> <rcLJ> <dt> <n>\n", argv[0]);
	return 2;
}
