// The `tc` mode of ref_harness.cpp: the reference's own TemperatureControl
// (thermostats/TemperatureControl), read from an XML file and driven the way
// Simulation::simulateOneTimestep drives it.  A separate translation unit
// because TemperatureControl.h declares a class Accumulator that clashes with
// utils/Accumulator.h of the ResultWriter mode.  Test infrastructure only.

#include <any>
#include <array>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <functional>
#include <list>
#include <map>
#include <memory>
#include <numeric>
#include <optional>
#include <set>
#include <sstream>
#include <string>
#include <tuple>
#include <unordered_map>
#include <utility>
#include <variant>
#include <vector>
#define private public
#include "Simulation.h"
#include "thermostats/TemperatureControl.h"
#undef private
#include "parallel/DomainDecompBase.h"
#include "particleContainer/ParticleContainer.h"
#include "utils/xmlfileUnits.h"

// TemperatureControl::readXML + prepare_start on the <temperatureControl>
// element of the file (the Simulation of the loaded phase space supplies the
// box lengths of "box" corners).
void* harnessTcCreate(const char* xml) {
	XMLfileUnits cfg(xml);
	cfg.changecurrentnode("/temperatureControl");
	auto* tc = new TemperatureControl();
	tc->readXML(cfg);
	tc->prepare_start();
	return tc;
}

// DoLoopsOverMolecules for simulation step k (the regions' ramps read the
// simulation's step number), then one TCB record per slab of every region
// that measured in this step: <k> <region> <slab> <beta_trans> <beta_rot> <N>.
void harnessTcStep(void* p, DomainDecompBase* dd, ParticleContainer* lc, unsigned long k) {
	auto* tc = static_cast<TemperatureControl*>(p);
	global_simulation->_simstep = k;
	std::vector<unsigned long> sampled;
	for (auto* reg : tc->_vecControlRegions) sampled.push_back(reg->_numSampledConfigs);
	tc->DoLoopsOverMolecules(dd, lc, k);
	for (size_t r = 0; r < tc->_vecControlRegions.size(); ++r) {
		ControlRegionT* reg = tc->_vecControlRegions[r];
		if (reg->_numSampledConfigs == sampled[r]) continue;  // no measurement in this step
		for (size_t b = 0; b < reg->_globalThermVars.size(); ++b)
			std::printf("TCB %lu %zu %zu %.17g %.17g %lu\n", k, r, b, reg->_globalThermVars[b]._betaTrans,
						reg->_globalThermVars[b]._betaRot, reg->_globalThermVars[b]._numMolecules);
	}
}
