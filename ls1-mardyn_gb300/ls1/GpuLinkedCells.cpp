/*
 * GpuLinkedCells.cpp -- see GpuLinkedCells.h.
 */
#include "GpuLinkedCells.h"

#include <sstream>

#if defined(_OPENMP)
#include <omp.h>
#endif

#include "Domain.h"
#include "Simulation.h"
#include "ensemble/EnsembleBase.h"
#include "molecules/Component.h"
#include "molecules/mixingrules/MixingRuleBase.h"
#include "particleContainer/adapter/CellProcessor.h"
#include "utils/Logger.h"
#include "utils/mardyn_assert.h"
#include "utils/xmlfileUnits.h"

GpuLinkedCells::GpuLinkedCells(double bBoxMin[3], double bBoxMax[3], double cutoffRadius)
	: LinkedCells(bBoxMin, bBoxMax, cutoffRadius) {}

GpuLinkedCells::~GpuLinkedCells() {
	if (_ctx) md_destroy(_ctx);
}

void GpuLinkedCells::check(int rc, const char* what) const {
	if (rc != MD_OK) {
		std::ostringstream msg;
		msg << "GpuLinkedCells: " << what << " failed (" << rc << "): " << md_last_error(_ctx) << std::endl;
		MARDYN_EXIT(msg.str());
	}
}

void GpuLinkedCells::readXML(XMLfileUnits& xmlconfig) {
	LinkedCells::readXML(xmlconfig);
	std::string prec = "mixed";
	xmlconfig.getNodeValue("precision", prec);
	_precision = (prec == "fp64") ? MD_PREC_FP64 : MD_PREC_MIXED;
	xmlconfig.getNodeValueReduced("skin", _skin);
	xmlconfig.getNodeValue("device", _device);
	std::string scheme = "rows";
	xmlconfig.getNodeValue("pairscheme", scheme);
	_pairScheme = (scheme == "newton3") ? MD_PAIRS_NEWTON3 : MD_PAIRS_ROWS;
	Log::global_log->info() << "GpuLinkedCells: precision " << prec << ", skin " << _skin << ", device " << _device
							<< ", pair scheme " << scheme << std::endl;
}

void GpuLinkedCells::update() {
	if (_ctx && !_deviceStale) return;  // the device re-bins itself
	LinkedCells::update();
}

void GpuLinkedCells::updateMoleculeCaches() {
	if (_ctx && !_deviceStale) return;  // site caches live on the device
	LinkedCells::updateMoleculeCaches();
}

void GpuLinkedCells::deleteOuterParticles() {
	if (_ctx && !_deviceStale) return;  // the halo exists on the device only
	LinkedCells::deleteOuterParticles();
}

void GpuLinkedCells::ensureDevice() {
	if (!_ctx) {
		md_config cfg{};
		for (int d = 0; d < 3; ++d) {
			cfg.box_min[d] = getBoundingBoxMin(d);
			cfg.box_max[d] = getBoundingBoxMax(d);
			cfg.periodic[d] = 1;  // serial DomainDecompBase: periodic halo in every dimension
		}
		cfg.rc = _rc;
		cfg.rc_lj = _rcLJ;
		cfg.eps_rf = global_simulation->getDomain()->getepsilonRF();
		cfg.precision = _precision;
		cfg.skin = _skin;
		cfg.device = _device;
		cfg.pair_scheme = _pairScheme;
		check(md_create(&_ctx, &cfg), "md_create");
		// components and Lorentz-Berthelot coefficients (Comp2Param::initialize inputs)
		std::vector<Component>& comps = *(global_simulation->getEnsemble()->getComponents());
		std::vector<std::vector<double>> tables(4 * comps.size());
		std::vector<md_component> mc(comps.size());
		for (size_t c = 0; c < comps.size(); ++c) {
			Component& C = comps[c];
			auto& lj = tables[4 * c];
			for (unsigned i = 0; i < C.numLJcenters(); ++i) {
				const LJcenter& s = C.ljcenter(i);
				lj.insert(lj.end(), {s.rx(), s.ry(), s.rz(), s.m(), s.eps(), s.sigma(), s.shift6()});
			}
			auto& ch = tables[4 * c + 1];
			for (unsigned i = 0; i < C.numCharges(); ++i) {
				const Charge& s = C.charge(i);
				ch.insert(ch.end(), {s.rx(), s.ry(), s.rz(), s.m(), s.q()});
			}
			auto& di = tables[4 * c + 2];
			for (unsigned i = 0; i < C.numDipoles(); ++i) {
				const Dipole& s = C.dipole(i);
				di.insert(di.end(), {s.rx(), s.ry(), s.rz(), s.ex(), s.ey(), s.ez(), s.abs()});
			}
			auto& qu = tables[4 * c + 3];
			for (unsigned i = 0; i < C.numQuadrupoles(); ++i) {
				const Quadrupole& s = C.quadrupole(i);
				qu.insert(qu.end(), {s.rx(), s.ry(), s.rz(), s.ex(), s.ey(), s.ez(), s.abs()});
			}
			mc[c].n_lj = (int32_t)C.numLJcenters();
			mc[c].n_charge = (int32_t)C.numCharges();
			mc[c].n_dipole = (int32_t)C.numDipoles();
			mc[c].n_quadrupole = (int32_t)C.numQuadrupoles();
			mc[c].lj = tables[4 * c].data();
			mc[c].charge = tables[4 * c + 1].data();
			mc[c].dipole = tables[4 * c + 2].data();
			mc[c].quadrupole = tables[4 * c + 3].data();
			// principal moments as the component holds them (header overrides included)
			mc[c].inertia[0] = C.I11();
			mc[c].inertia[1] = C.I22();
			mc[c].inertia[2] = C.I33();
		}
		std::vector<double> mixing;
		auto& rules = global_simulation->getEnsemble()->getMixingrules();
		for (size_t i = 0; i < comps.size(); ++i)
			for (size_t j = i + 1; j < comps.size(); ++j) {
				const auto p = rules.at(i).at(j)->getParameters();  // (eta, xi) of the LB rule
				mixing.push_back(p.at(1));
				mixing.push_back(p.at(0));
			}
		check(md_set_components(_ctx, mc.data(), (int32_t)mc.size(), mixing.empty() ? nullptr : mixing.data()),
			  "md_set_components");
	}
	if (_deviceStale) upload();
}

void GpuLinkedCells::upload() {
	std::vector<uint64_t> id;
	std::vector<int32_t> comp;
	std::vector<double> r, v, q, L, F, M, Vi;
	_ids.clear();
	_slot.clear();
	for (auto m = LinkedCells::iterator(ParticleIterator::ONLY_INNER_AND_BOUNDARY); m.isValid(); ++m) {
		_slot[m->getID()] = _ids.size();
		_ids.push_back(m->getID());
		id.push_back(m->getID());
		comp.push_back((int32_t)m->componentid());
		for (int d = 0; d < 3; ++d) {
			r.push_back(m->r(d));
			v.push_back(m->v(d));
			L.push_back(m->D(d));
		}
		const Quaternion qq = m->q();
		q.insert(q.end(), {qq.qw(), qq.qx(), qq.qy(), qq.qz()});
		for (int d = 0; d < 3; ++d) {
			F.push_back(m->F(d));
			M.push_back(m->M(d));
			Vi.push_back(m->Vi(d));
		}
	}
	check(md_upload_molecules(_ctx, (int64_t)id.size(), id.data(), comp.data(), r.data(), v.data(), q.data(),
							  L.data()),
		  "md_upload_molecules");
	// the next pre-force half step kicks with these (the upload clears the device's)
	check(md_set_forces(_ctx, (int64_t)id.size(), F.data(), M.data(), Vi.data()), "md_set_forces");
	_deviceStale = false;
	_hostStale = false;
}

// The device state into host buffers (upload order).
void GpuLinkedCells::downloadState() {
	const size_t n = _ids.size();
	for (auto* b : {&_dr, &_dv, &_dL, &_dF, &_dM, &_dVi}) b->resize(3 * n);
	_dq.resize(4 * n);
	check(md_download_molecules(_ctx, (int64_t)n, nullptr, nullptr, _dr.data(), _dv.data(), _dq.data(), _dL.data(),
								_dF.data(), _dM.data(), _dVi.data()),
		  "md_download_molecules");
}

// The downloaded values into the mirror molecules the container's iterator
// hands this thread (all of them outside a parallel region), copies of which
// go to `out`.
void GpuLinkedCells::applyDownload(std::vector<Molecule>& out) {
	for (auto m = LinkedCells::iterator(ParticleIterator::ONLY_INNER_AND_BOUNDARY); m.isValid(); ++m) {
		const size_t k = _slot.at(m->getID());
		for (int d = 0; d < 3; ++d) {
			m->setr(d, _dr[3 * k + d]);
			m->setv(d, _dv[3 * k + d]);
			m->setD(d, _dL[3 * k + d]);
		}
		m->setq(Quaternion(_dq[4 * k], _dq[4 * k + 1], _dq[4 * k + 2], _dq[4 * k + 3]));
		m->setF(&_dF[3 * k]);
		m->setM(&_dM[3 * k]);
		m->setVi(&_dVi[3 * k]);
		out.push_back(*m);
	}
}

// Re-bin the mirror from scratch: since the last sync a molecule may have
// crossed a periodic boundary on the device (its position wrapped to the far
// side), which LinkedCells::update, built for moves of at most one cell, does
// not handle; the halo cells stay empty until the host rebuilds them.
void GpuLinkedCells::rebinMirror(std::vector<Molecule>& mols) {
	LinkedCells::clear();
	LinkedCells::addParticles(mols);
	mols.clear();
	_hostStale = false;
	_deviceStale = true;  // the caller may now edit molecules through the iterator
}

void GpuLinkedCells::syncToHost() {
	if (!_ctx || !_hostStale) return;
	downloadState();
	std::vector<Molecule> mols;
	mols.reserve(_ids.size());
	applyDownload(mols);
	rebinMirror(mols);
}

// ls1 iterates the container inside OpenMP parallel regions, every thread of
// the team asking for its own iterator, which covers that thread's share of
// the cells (e.g. Leapfrog.cpp:84-125, Domain.cpp:457-480): the download is
// done by one thread, every thread then updates its share of the mirror, and
// one thread re-bins it; the barriers keep the team from iterating a mirror
// that is not complete.
void GpuLinkedCells::syncForIteration() {
#if defined(_OPENMP)
	if (omp_in_parallel()) {
		bool need = false;
		#pragma omp single copyprivate(need)
		{
			need = _ctx != nullptr && _hostStale;
			if (need) downloadState();
		}
		if (!need) return;
		std::vector<Molecule> mine;
		applyDownload(mine);
		#pragma omp critical(gpu_linked_cells_sync)
		_pending.insert(_pending.end(), mine.begin(), mine.end());
		#pragma omp barrier
		#pragma omp single
		rebinMirror(_pending);
		return;
	}
#endif
	syncToHost();
}

md_ctx* GpuLinkedCells::deviceContext() {
	ensureDevice();
	return _ctx;
}

void GpuLinkedCells::traverseCells(CellProcessor& cellProcessor) {
	if (!_ctx) {
		_rc = cellProcessor.getCutoffRadius();
		_rcLJ = cellProcessor.getLJCutoffRadius();
	}
	ensureDevice();
	md_forces_out out{};
	check(md_compute_forces(_ctx, &out), "md_compute_forces");
	// VectorizedCellProcessor::endTraversal hands these to the domain
	global_simulation->getDomain()->setLocalVirial(out.virial);
	global_simulation->getDomain()->setLocalUpot(out.upot);
	_hostStale = true;
}

ParticleIterator GpuLinkedCells::iterator(ParticleIterator::Type t) {
	syncForIteration();
	return LinkedCells::iterator(t);
}

RegionParticleIterator GpuLinkedCells::regionIterator(const double startCorner[3], const double endCorner[3],
													  ParticleIterator::Type t) {
	syncForIteration();
	return LinkedCells::regionIterator(startCorner, endCorner, t);
}

unsigned long GpuLinkedCells::getNumberOfParticles(ParticleIterator::Type t) {
	if (_ctx && !_deviceStale && t != ParticleIterator::ALL_CELLS) return _ids.size();
	return LinkedCells::getNumberOfParticles(t);
}
