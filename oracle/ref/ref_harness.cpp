// Test-infrastructure driver around the reference implementation's own
// short-range MD path.  It is linked against the reference's objects (built
// from its sources by the Makefile beside it) and only prints what the
// reference computes; it implements no physics of its own.
//
// Modes (all values printed with 17 significant digits):
//   forces <file.inp> <rc> <rcLJ> <periodic 0|1>
//       One force evaluation, set up the way the reference's unit tests do
//       (ParticleContainerFactory::createInitializedParticleContainer): read the
//       ASCII phase space, build LinkedCells(cutoff = rc), update, optionally
//       run the serial periodic exchange (leaving particles + halo copies),
//       build the SoA caches, traverse with VectorizedCellProcessor and call
//       calcFM on every inner molecule.  Also traverses with the FlopCounter.
//   nvt <file.inp> <rc> <rcLJ> <dt> <nsteps> <T>
//       As `steps`, with the global velocity-scaling thermostat at target T:
//       after the global values of each step, v *= beta_trans and
//       D *= beta_rot (Simulation::simulateOneTimestep, VELSCALE_THERMOSTAT
//       with one thermostat).  STEP records carry the values before scaling
//       and a BETA record follows each.
//   nvtc <file.inp> <rc> <rcLJ> <dt> <nsteps> <T_1> ... <T_ncomp>
//       As `nvt` with a component-wise thermostat: component c on thermostat
//       c+1 with target T_{c+1} (Domain::setComponentThermostat /
//       setTargetTemperature), the velocity scaling of
//       Simulation::simulateOneTimestep's several-thermostats branch.  BETA
//       records carry <k> <thermostat> <beta_trans> <beta_rot>.
//   lrc <file.inp> <rc> <rcLJ>
//       The homogeneous long-range correction (longRange/Homogeneous): init +
//       calculateLongRange, then the global values with zero local Upot and
//       virial, so the printed global Upot and virial are the corrections.
//   binw <file.inp> <rc> <prefix> <time>
//       Domain::writeCheckpoint with the binary format (the CheckpointWriter's
//       `binary` type): <prefix>.header.xml (writeCheckpointHeaderXML) and
//       <prefix>.dat (FullMolecule::writeBinary of every molecule in container
//       order).
//   binr <components.inp> <header.xml> <data> <rc>
//       Components and box from the ASCII file's header, then BinaryReader:
//       readPhaseSpaceHeader + readPhaseSpace; prints the molecules read.
//   planar <file.inp> <rc> <rcLJ> <dt> <nsteps> <slabs> <frequency> <y_lo> <y_hi>
//       As `steps`, with the planar long-range correction (longRange/Planar)
//       in the place Simulation gives it: after the traversal and before
//       calcFM, at the first force evaluation and in every step; force
//       corrections applied to molecules with y in [y_lo, y_hi].  LRC
//       records carry the step's UpotCorr and VirialCorr.
//   res <file.inp> <rc> <rcLJ> <dt> <nsteps> <T> <prefix> <writefrequency> <accumulation_steps> <writeprecision>
//       As `nvt` (T > 0) or `steps` (T = 0), with the reference's ResultWriter
//       (io/ResultWriter.cpp) set up as its readXML would with these values:
//       init() before the first step, endStep() after each step's global
//       values and thermostat, the simulation time advanced by dt each step
//       as Simulation::simulateOneTimestep does; writes <prefix>.res.
//   tc <file.inp> <rc> <rcLJ> <dt> <nsteps> <tc.xml>
//       As `steps`, with the reference's TemperatureControl read from the
//       <temperatureControl> element of tc.xml (TemperatureControl::readXML,
//       prepare_start) and DoLoopsOverMolecules(simstep = k) after each
//       step's global values, where Simulation::simulateOneTimestep calls it.
//       TCB records carry <k> <region> <slab> <beta_trans> <beta_rot> <N>
//       after each measuring step.  Writes the reference's beta and added
//       kinetic energy logs into the working directory.
//   steps <file.inp> <rc> <rcLJ> <dt> <nsteps>
//       NVE Leapfrog steps with the periodic halo, in the order of the
//       reference's Simulation::simulateOneTimestep (thermostat off, no
//       long-range correction).  Prints per-step Upot, virial, 2*Ukin_trans and
//       2*Ukin_rot and the final per-molecule state.
//
// Output records:
//   N <count>
//   GRID <cells per dim incl. halo x3> <cell length x3>
//   UPOT <local Upot>   VIRIAL <local virial>
//   COUNTS <molecule distances> {<kernel calls> <macro calls>} x 7 potentials
//   STEP <k> <Upot> <virial> <summv2> <sumIw2>
//   LRC <UpotCorr> <VirialCorr>
//   BETA <k> <beta_trans> <beta_rot>
//   MOL <id> <comp> <cell> r[3] v[3] q[4] L[3] F[3] M[3] Vi[3]

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>
#include <algorithm>
#include <iostream>
#include <memory>

// Simulation's particle-container pointer is private; the long-range mode
// points it at the harness's LinkedCells (the reference's Domain fetches the
// molecule count through it).  Standard headers are included first so that
// only the reference's own classes are opened.
#include <any>
#include <array>
#include <chrono>
#include <cmath>
#include <fstream>
#include <functional>
#include <list>
#include <map>
#include <optional>
#include <random>
#include <set>
#include <sstream>
#include <stack>
#include <tuple>
#include <unordered_map>
#include <utility>
#include <variant>
#include <iomanip>
#include <mutex>
#include <thread>
#include <limits>
#include <numeric>
#include <bitset>
#include <deque>
#include <queue>
#include <cstring>
#include <omp.h>
#define private public
#include "Simulation.h"
#include "Domain.h"
#include "longRange/Planar.h"
#include "io/ResultWriter.h"
#undef private
#include "ensemble/EnsembleBase.h"
#include "integrators/Leapfrog.h"
#include "io/ASCIIReader.h"
#include "io/BinaryReader.h"
#include "longRange/Homogeneous.h"
#include "thermostats/VelocityScalingThermostat.h"
#include "molecules/Molecule.h"
#include "parallel/DomainDecompBase.h"
#include "particleContainer/LinkedCells.h"
#include "particleContainer/adapter/VectorizedCellProcessor.h"
#include "particleContainer/adapter/vectorization/SIMD_TYPES.h"
#include "utils/Logger.h"
// The per-potential call counters of FlopCounter are private members; they are
// read here (not modified) to report the reference's own pair counts.
#define private public
#include "particleContainer/adapter/FlopCounter.h"
#undef private

static_assert(VCP_VEC_TYPE == VCP_NOVEC, "golden vectors come from the scalar kernel path");

// TemperatureControl lives in ref_harness_tc.cpp: its header declares a class
// Accumulator that clashes with the ResultWriter's utils/Accumulator.h.
void* harnessTcCreate(const char* xml);
void harnessTcStep(void* tc, DomainDecompBase* dd, ParticleContainer* lc, unsigned long k);

namespace {

struct Setup {
	Domain* domain = nullptr;
	DomainDecompBase* dd = nullptr;
	LinkedCells* lc = nullptr;
	ASCIIReader reader;
};

void load(Setup& s, const std::string& file, double rc, double rcLJ) {
	new Simulation();  // assigns global_simulation
	s.domain = global_simulation->getDomain();
	s.dd = &global_simulation->domainDecomposition();
	global_simulation->setcutoffRadius(rc);
	global_simulation->setLJCutoff(rcLJ);
	s.reader.setPhaseSpaceHeaderFile(file);
	s.reader.setPhaseSpaceFile(file);
	s.reader.readPhaseSpaceHeader(s.domain, 1.0);
	double bmin[3], bmax[3];
	for (int d = 0; d < 3; ++d) {
		bmin[d] = s.dd->getBoundingBoxMin(d, s.domain);
		bmax[d] = s.dd->getBoundingBoxMax(d, s.domain);
	}
	s.lc = new LinkedCells(bmin, bmax, rc);
	s.reader.readPhaseSpace(s.lc, s.domain, s.dd);
	s.lc->deleteOuterParticles();
	s.lc->update();
}

void printGrid(const Setup& s) {
	double bmin[3], bmax[3];
	for (int d = 0; d < 3; ++d) {
		bmin[d] = s.lc->getBoundingBoxMin(d);
		bmax[d] = s.lc->getBoundingBoxMax(d);
	}
	const double* cl = s.lc->getCellLength();
	int n[3];
	for (int d = 0; d < 3; ++d) n[d] = (int)((bmax[d] - bmin[d]) / cl[d] + 0.5) + 2;
	std::printf("GRID %d %d %d %.17g %.17g %.17g\n", n[0], n[1], n[2], cl[0], cl[1], cl[2]);
}

void printMolecules(Setup& s) {
	struct Row { unsigned long id; std::vector<double> v; int comp; unsigned long cell; };
	std::vector<Row> rows;
	for (auto m = s.lc->iterator(ParticleIterator::ONLY_INNER_AND_BOUNDARY); m.isValid(); ++m) {
		Row r;
		r.id = m->getID();
		r.comp = (int)m->componentid();
		r.cell = s.lc->getCellIndexOfMolecule(&(*m));
		const Quaternion q = m->q();
		const double vals[] = {m->r(0), m->r(1), m->r(2), m->v(0), m->v(1), m->v(2),
							   q.qw(), q.qx(), q.qy(), q.qz(), m->D(0), m->D(1), m->D(2),
							   m->F(0), m->F(1), m->F(2), m->M(0), m->M(1), m->M(2),
							   m->Vi(0), m->Vi(1), m->Vi(2)};
		r.v.assign(vals, vals + sizeof(vals) / sizeof(vals[0]));
		rows.push_back(r);
	}
	std::sort(rows.begin(), rows.end(), [](const Row& a, const Row& b) { return a.id < b.id; });
	std::printf("N %zu\n", rows.size());
	for (const Row& r : rows) {
		std::printf("MOL %lu %d %lu", r.id, r.comp, r.cell);
		for (double x : r.v) std::printf(" %.17g", x);
		std::printf("\n");
	}
}

int runForces(const std::string& file, double rc, double rcLJ, bool periodic) {
	Setup s;
	load(s, file, rc, rcLJ);
	if (periodic) s.dd->exchangeMolecules(s.lc, s.domain);
	s.lc->updateMoleculeCaches();
	s.domain->initParameterStreams(rc, rcLJ);

	FlopCounter flops(rc, rcLJ);
	s.lc->traverseCells(flops);

	VectorizedCellProcessor vcp(*s.domain, rc, rcLJ);
	s.lc->traverseCells(vcp);
	for (auto m = s.lc->iterator(ParticleIterator::ALL_CELLS); m.isValid(); ++m) m->calcFM();

	printGrid(s);
	std::printf("UPOT %.17g\nVIRIAL %.17g\n", s.domain->getLocalUpot(), s.domain->getLocalVirial());
	const auto& c = flops._currentCounts;
	std::printf("COUNTS %.17g", c._moleculeDistances);
	for (int i = 0; i < FlopCounter::NUM_POTENTIALS; ++i)
		std::printf(" %.17g %.17g", c._potCounts[i]._numKernelCalls, c._potCounts[i]._numMacroCalls);
	std::printf("\n");
	s.lc->deleteOuterParticles();
	printMolecules(s);
	return 0;
}

void forceStep(Setup& s, VectorizedCellProcessor& vcp) {
	s.lc->traverseCells(vcp);
	for (auto m = s.lc->iterator(ParticleIterator::ALL_CELLS); m.isValid(); ++m) m->calcFM();
	s.lc->deleteOuterParticles();
}

int runSteps(const std::string& file, double rc, double rcLJ, double dt, int nsteps, double T = 0.0,
			 ResultWriter* rw = nullptr, const char* tcXml = nullptr) {
	Setup s;
	load(s, file, rc, rcLJ);
	void* tc = tcXml ? harnessTcCreate(tcXml) : nullptr;
	if (T > 0.0) {
		s.domain->thermostatOn();
		s.domain->setGlobalTemperature(T);
	} else {
		s.domain->thermostatOff();
	}
	VelocityScalingThermostat thermostat;
	s.dd->exchangeMolecules(s.lc, s.domain);
	s.lc->updateMoleculeCaches();
	s.domain->initParameterStreams(rc, rcLJ);
	VectorizedCellProcessor vcp(*s.domain, rc, rcLJ);
	Leapfrog integrator(dt);

	// initial forces, as in Simulation::prepare_start
	forceStep(s, vcp);
	printGrid(s);
	std::printf("STEP 0 %.17g %.17g nan nan\n", s.domain->getLocalUpot(), s.domain->getLocalVirial());
	if (rw) {
		global_simulation->_moleculeContainer = s.lc;  // the Domain counts molecules through it
		s.domain->evaluateRho(s.lc->getNumberOfParticles(), s.dd);
		rw->init(s.lc, s.dd, s.domain);
	}
	for (int k = 1; k <= nsteps; ++k) {
		integrator.eventNewTimestep(s.lc, s.domain);
		s.lc->update();
		s.dd->exchangeMolecules(s.lc, s.domain);
		s.lc->updateMoleculeCaches();
		forceStep(s, vcp);
		integrator.eventForcesCalculated(s.lc, s.domain);
		const double upot = s.domain->getLocalUpot();
		const double vir = s.domain->getLocalVirial();
		s.domain->calculateGlobalValues(s.dd, s.lc, false, 1.0);
		std::printf("STEP %d %.17g %.17g %.17g %.17g\n", k, upot, vir,
					2.0 * s.domain->getGlobalUkinTrans(), 2.0 * s.domain->getGlobalUkinRot());
		if (T > 0.0) {
			thermostat.setGlobalBetaTrans(s.domain->getGlobalBetaTrans());
			thermostat.setGlobalBetaRot(s.domain->getGlobalBetaRot());
			thermostat.apply(s.lc);
			std::printf("BETA %d %.17g %.17g\n", k, s.domain->getGlobalBetaTrans(), s.domain->getGlobalBetaRot());
		}
		if (tc) harnessTcStep(tc, s.dd, s.lc, (unsigned long)k);
		if (rw) {
			global_simulation->advanceSimulationTime(dt);  // Simulation::simulateOneTimestep, before the plugins' endStep
			rw->endStep(s.lc, s.dd, s.domain, (unsigned long)k);
		}
	}
	printMolecules(s);
	return 0;
}

// ResultWriter::readXML's settings without an XML file.
int runResults(const std::string& file, double rc, double rcLJ, double dt, int nsteps, double T,
			   const std::string& prefix, int freq, int acc, int precision) {
	ResultWriter rw;
	rw._writeFrequency = freq;
	rw._outputPrefix = prefix;
	rw._U_pot_acc = std::make_unique<Accumulator<double>>(acc);
	rw._U_kin_acc = std::make_unique<Accumulator<double>>(acc);
	rw._p_acc = std::make_unique<Accumulator<double>>(acc);
	rw._writePrecision = precision;
	rw._writeWidth = precision + 15;
	return runSteps(file, rc, rcLJ, dt, nsteps, T, &rw);
}

int runPlanar(const std::string& file, double rc, double rcLJ, double dt, int nsteps, int slabs, int freq,
			  double ylo, double yhi) {
	Setup s;
	load(s, file, rc, rcLJ);
	s.domain->thermostatOff();
	s.dd->exchangeMolecules(s.lc, s.domain);
	s.lc->updateMoleculeCaches();
	s.domain->initParameterStreams(rc, rcLJ);
	global_simulation->_moleculeContainer = s.lc;
	VectorizedCellProcessor vcp(*s.domain, rc, rcLJ);
	Leapfrog integrator(dt);
	Planar lrc(rc, rcLJ, s.domain, s.dd, s.lc, (unsigned)slabs, global_simulation);
	lrc.frequency = freq;
	lrc._region.refPosID[0] = lrc._region.refPosID[1] = 0;
	lrc._region.refPos[0] = lrc._region.actPos[0] = ylo;
	lrc._region.refPos[1] = lrc._region.actPos[1] = yhi;
	lrc.init();
	auto forcesWithLrc = [&]() {
		s.lc->traverseCells(vcp);
		lrc.calculateLongRange();
		for (auto m = s.lc->iterator(ParticleIterator::ALL_CELLS); m.isValid(); ++m) m->calcFM();
		s.lc->deleteOuterParticles();
		std::printf("LRC %.17g %.17g\n", s.domain->_UpotCorr, s.domain->_VirialCorr);
	};
	forcesWithLrc();
	std::printf("STEP 0 %.17g %.17g nan nan\n", s.domain->getLocalUpot(), s.domain->getLocalVirial());
	for (int k = 1; k <= nsteps; ++k) {
		integrator.eventNewTimestep(s.lc, s.domain);
		s.lc->update();
		s.dd->exchangeMolecules(s.lc, s.domain);
		s.lc->updateMoleculeCaches();
		forcesWithLrc();
		integrator.eventForcesCalculated(s.lc, s.domain);
		const double upot = s.domain->getLocalUpot();
		const double vir = s.domain->getLocalVirial();
		s.domain->calculateGlobalValues(s.dd, s.lc, false, 1.0);
		std::printf("STEP %d %.17g %.17g %.17g %.17g\n", k, upot, vir, 2.0 * s.domain->getGlobalUkinTrans(),
					2.0 * s.domain->getGlobalUkinRot());
	}
	printMolecules(s);
	return 0;
}

int runNvtComponentwise(const std::string& file, double rc, double rcLJ, double dt, int nsteps,
						const std::vector<double>& T) {
	Setup s;
	load(s, file, rc, rcLJ);
	s.domain->thermostatOn();
	const int ncomp = (int)global_simulation->getEnsemble()->getComponents()->size();
	for (int c = 0; c < ncomp; ++c) s.domain->setComponentThermostat(c, c + 1);
	for (int c = 0; c < ncomp; ++c) s.domain->setTargetTemperature(c + 1, T[c]);
	VelocityScalingThermostat thermostat;
	s.dd->exchangeMolecules(s.lc, s.domain);
	s.lc->updateMoleculeCaches();
	s.domain->initParameterStreams(rc, rcLJ);
	VectorizedCellProcessor vcp(*s.domain, rc, rcLJ);
	Leapfrog integrator(dt);
	forceStep(s, vcp);
	std::printf("STEP 0 %.17g %.17g nan nan\n", s.domain->getLocalUpot(), s.domain->getLocalVirial());
	for (int k = 1; k <= nsteps; ++k) {
		integrator.eventNewTimestep(s.lc, s.domain);
		s.lc->update();
		s.dd->exchangeMolecules(s.lc, s.domain);
		s.lc->updateMoleculeCaches();
		forceStep(s, vcp);
		integrator.eventForcesCalculated(s.lc, s.domain);
		const double upot = s.domain->getLocalUpot();
		const double vir = s.domain->getLocalVirial();
		s.domain->calculateGlobalValues(s.dd, s.lc, false, 1.0);
		std::printf("STEP %d %.17g %.17g %.17g %.17g\n", k, upot, vir, 2.0 * s.domain->getGlobalUkinTrans(),
					2.0 * s.domain->getGlobalUkinRot());
		thermostat.enableComponentwise();
		for (int c = 0; c < ncomp; ++c) {
			const int tid = s.domain->getThermostat(c);
			thermostat.setBetaTrans(tid, s.domain->getGlobalBetaTrans(tid));
			thermostat.setBetaRot(tid, s.domain->getGlobalBetaRot(tid));
			double v[3];
			for (int d = 0; d < 3; d++) v[d] = s.domain->getThermostatDirectedVelocity(tid, d);
			thermostat.setVelocity(tid, v);
			std::printf("BETA %d %d %.17g %.17g\n", k, tid, s.domain->getGlobalBetaTrans(tid),
						s.domain->getGlobalBetaRot(tid));
		}
		thermostat.apply(s.lc);
	}
	printMolecules(s);
	return 0;
}

int runLrc(const std::string& file, double rc, double rcLJ) {
	Setup s;
	load(s, file, rc, rcLJ);
	s.domain->thermostatOff();
	s.domain->initParameterStreams(rc, rcLJ);
	global_simulation->_moleculeContainer = s.lc;
	Homogeneous lrc(rc, rcLJ, s.domain, s.lc, global_simulation);
	lrc.init();
	lrc.calculateLongRange();
	s.domain->setLocalUpot(0.0);
	s.domain->setLocalVirial(0.0);
	s.domain->calculateGlobalValues(s.dd, s.lc, false, 1.0);
	const double n = (double)s.domain->getglobalNumMolecules(false);
	std::printf("LRC %.17g %.17g\n", s.domain->getGlobalUpot(), s.domain->getAverageGlobalVirial() * n);
	return 0;
}

int runBinWrite(const std::string& file, double rc, const std::string& prefix, double time) {
	Setup s;
	load(s, file, rc, rc);
	s.domain->writeCheckpoint(prefix, s.lc, s.dd, time, true);
	std::printf("N %lu\n", s.domain->getglobalNumMolecules(true, s.lc, s.dd));
	return 0;
}

int runBinRead(const std::string& inp, const std::string& header, const std::string& data, double rc) {
	Setup s;
	new Simulation();
	s.domain = global_simulation->getDomain();
	s.dd = &global_simulation->domainDecomposition();
	global_simulation->setcutoffRadius(rc);
	global_simulation->setLJCutoff(rc);
	s.reader.setPhaseSpaceHeaderFile(inp);
	s.reader.readPhaseSpaceHeader(s.domain, 1.0);
	BinaryReader br;
	br.setPhaseSpaceHeaderFile(header);
	br.setPhaseSpaceFile(data);
	br.readPhaseSpaceHeader(s.domain, 1.0);
	double bmin[3], bmax[3];
	for (int d = 0; d < 3; ++d) {
		bmin[d] = s.dd->getBoundingBoxMin(d, s.domain);
		bmax[d] = s.dd->getBoundingBoxMax(d, s.domain);
	}
	s.lc = new LinkedCells(bmin, bmax, rc);
	br.readPhaseSpace(s.lc, s.domain, s.dd);
	std::printf("TIME %.17g\nLENGTH %.17g %.17g %.17g\n", global_simulation->getSimulationTime(),
				s.domain->getGlobalLength(0), s.domain->getGlobalLength(1), s.domain->getGlobalLength(2));
	printMolecules(s);
	return 0;
}

}  // namespace

int main(int argc, char** argv) {
	// The reference logs through a global logger that its own main() creates;
	// send it to stderr so stdout carries only the records above.
	Log::global_log = std::make_unique<Log::Logger>(Log::Warning, std::shared_ptr<std::ostream>(&std::cerr, [](void*) {}));
	if (argc >= 6 && std::string(argv[1]) == "forces")
		return runForces(argv[2], std::atof(argv[3]), std::atof(argv[4]), std::atoi(argv[5]) != 0);
	if (argc >= 8 && std::string(argv[1]) == "nvt")
		return runSteps(argv[2], std::atof(argv[3]), std::atof(argv[4]), std::atof(argv[5]), std::atoi(argv[6]),
						std::atof(argv[7]));
	if (argc >= 8 && std::string(argv[1]) == "nvtc") {
		std::vector<double> T;
		for (int a = 7; a < argc; ++a) T.push_back(std::atof(argv[a]));
		return runNvtComponentwise(argv[2], std::atof(argv[3]), std::atof(argv[4]), std::atof(argv[5]),
								   std::atoi(argv[6]), T);
	}
	if (argc >= 5 && std::string(argv[1]) == "lrc")
		return runLrc(argv[2], std::atof(argv[3]), std::atof(argv[4]));
	if (argc >= 11 && std::string(argv[1]) == "planar")
		return runPlanar(argv[2], std::atof(argv[3]), std::atof(argv[4]), std::atof(argv[5]), std::atoi(argv[6]),
						 std::atoi(argv[7]), std::atoi(argv[8]), std::atof(argv[9]), std::atof(argv[10]));
	if (argc >= 6 && std::string(argv[1]) == "binw")
		return runBinWrite(argv[2], std::atof(argv[3]), argv[4], std::atof(argv[5]));
	if (argc >= 6 && std::string(argv[1]) == "binr")
		return runBinRead(argv[2], argv[3], argv[4], std::atof(argv[5]));
	if (argc >= 12 && std::string(argv[1]) == "res")
		return runResults(argv[2], std::atof(argv[3]), std::atof(argv[4]), std::atof(argv[5]), std::atoi(argv[6]),
						  std::atof(argv[7]), argv[8], std::atoi(argv[9]), std::atoi(argv[10]), std::atoi(argv[11]));
	if (argc >= 8 && std::string(argv[1]) == "tc")
		return runSteps(argv[2], std::atof(argv[3]), std::atof(argv[4]), std::atof(argv[5]), std::atoi(argv[6]), 0.0,
						nullptr, argv[7]);
	if (argc >= 7 && std::string(argv[1]) == "steps")
		return runSteps(argv[2], std::atof(argv[3]), std::atof(argv[4]), std::atof(argv[5]), std::atoi(argv[6]));
	std::fprintf(stderr, "usage: %s forces <inp> <rc> <rcLJ> <periodic> | lrc <inp> <rc> <rcLJ> | steps <inp> <rc> <rcLJ> <dt> <n> | nvt <inp> <rc> <rcLJ> <dt> <n> <T> | binw <inp> <rc> <prefix> <time> | binr <inp> <header> <data> <rc>\n", argv[0]);
	return 2;
}
