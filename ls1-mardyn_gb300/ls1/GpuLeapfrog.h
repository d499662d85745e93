/*
 * GpuLeapfrog.h -- ls1-MarDyn Integrator running Leapfrog on the device of a
 * GpuLinkedCells container (<integrator type="GpuLeapfrog">,
 * src/Simulation.cpp:171-195).  Same state machine and sums as Leapfrog
 * (src/integrators/Leapfrog.cpp:32-147): eventNewTimestep performs the
 * pre-force half step (upd_preF), eventForcesCalculated the post-force half
 * step (upd_postF) and hands sum m v^2, sum I w^2, N and the rotational
 * degrees of freedom to Domain for thermostat 0.
 */
#pragma once

#include "integrators/Integrator.h"

class GpuLeapfrog : public Integrator {
public:
	GpuLeapfrog() = default;
	explicit GpuLeapfrog(double timestepLength) { _timestepLength = timestepLength; }
	void readXML(XMLfileUnits& xmlconfig) override;
	void init() override {}
	void eventForcesCalculated(ParticleContainer* moleculeContainer, Domain* domain) override;
	void eventNewTimestep(ParticleContainer* moleculeContainer, Domain* domain) override;

private:
	bool _postForcePending = false;
};
