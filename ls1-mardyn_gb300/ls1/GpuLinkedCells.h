/*
 * GpuLinkedCells.h -- ls1-MarDyn ParticleContainer whose short-range path runs
 * on a GB300 through the ls1gb300 C ABI (include/ls1gb300.h).
 *
 * Drop-in beside LinkedCells (src/particleContainer/LinkedCells.h), selected
 * with <datastructure type="GpuLinkedCells"> (src/Simulation.cpp:471-515).
 * Like AutoPasContainer::traverseCells (src/particleContainer/AutoPasContainer.cpp:559-606)
 * it receives the VectorizedCellProcessor but only takes its cut-offs; the
 * forces, torques and per-molecule virials are computed on the device and
 * Upot/virial are handed to Domain as VectorizedCellProcessor::endTraversal
 * does (src/particleContainer/adapter/VectorizedCellProcessor.cpp:122-155).
 *
 * The host LinkedCells cells remain the molecule mirror that plugins, writers
 * and thermostats iterate.  Between traversals the device holds the
 * authoritative state; iterating the container downloads it (positions
 * wrapped into the box, the mirror re-binned) and marks the device copy for
 * re-upload, since a caller may modify molecules through the iterator.
 */
#pragma once

#include <string>
#include <unordered_map>
#include <vector>

#include "ls1gb300.h"
#include "particleContainer/LinkedCells.h"

class GpuLinkedCells : public LinkedCells {
public:
	GpuLinkedCells() = default;  // XML path: setCutoff + rebuild, as for LinkedCells
	GpuLinkedCells(double bBoxMin[3], double bBoxMax[3], double cutoffRadius);
	~GpuLinkedCells() override;

	/* <datastructure type="GpuLinkedCells">
	 *     <precision>mixed|fp64</precision>   (default mixed)
	 *     <skin>0.3</skin>                     (pair-candidate list skin, default 0.3)
	 *     <device>0</device>
	 * </datastructure> */
	void readXML(XMLfileUnits& xmlconfig) override;

	/* The device re-bins, rebuilds the halo and its site caches itself inside
	 * md_compute_forces / md_run; while it is authoritative the host mirror is
	 * left untouched. */
	void update() override;
	void updateMoleculeCaches() override;
	void deleteOuterParticles() override;

	void traverseCells(CellProcessor& cellProcessor) override;

	ParticleIterator iterator(ParticleIterator::Type t) override;
	RegionParticleIterator regionIterator(const double startCorner[3], const double endCorner[3],
										  ParticleIterator::Type t) override;
	unsigned long getNumberOfParticles(ParticleIterator::Type t = ParticleIterator::ALL_CELLS) override;
	std::string getName() override { return "GpuLinkedCells"; }
	/* Every pair's force reaches both molecules on the device (no force
	 * exchange of halo copies, ParticleContainer.h:232); LinkedCells would ask
	 * its traversal tuner, which never runs here. */
	bool requiresForceExchange() const override { return false; }

	/* Used by GpuLeapfrog: the device context (uploading the mirror first if
	 * it was edited) and the notice that the device state moved on. */
	md_ctx* deviceContext();
	void deviceStepped() { _hostStale = true; }
	/* true while the device holds the state: Simulation then skips the host
	 * rebin/halo exchange and the host calcFM (see Simulation.patch). */
	bool deviceAuthoritative() const { return _ctx != nullptr && !_deviceStale; }

private:
	void ensureDevice();
	void upload();
	void syncToHost();
	void syncForIteration();
	void downloadState();
	void applyDownload(std::vector<Molecule>& out);
	void rebinMirror(std::vector<Molecule>& mols);
	void check(int rc, const char* what) const;

	md_ctx* _ctx = nullptr;
	int _precision = MD_PREC_MIXED;
	double _skin = 0.3;
	int _device = 0;
	int _pairScheme = MD_PAIRS_ROWS;  // <pairscheme>rows|newton3</pairscheme>
	double _rc = 0.0, _rcLJ = 0.0;
	bool _hostStale = false;    // device state ahead of the host mirror
	bool _deviceStale = true;   // host mirror edited since the last upload
	std::vector<unsigned long> _ids;                 // upload order
	std::unordered_map<unsigned long, size_t> _slot; // id -> upload index
	std::vector<double> _dr, _dv, _dq, _dL, _dF, _dM, _dVi;  // the last download (upload order)
	std::vector<Molecule> _pending;                  // mirror molecules gathered by the team for the re-bin
};
