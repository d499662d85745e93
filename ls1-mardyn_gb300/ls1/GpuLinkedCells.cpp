/*
 * GpuLinkedCells.cpp -- see GpuLinkedCells.h.
 */
#include "GpuLinkedCells.h"

#include <sstream>

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
	Log::global_log->info() << "GpuLinkedCells: precision " << prec << ", skin " << _skin << ", device " << _device
							<< std::endl;
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
	std::vector<double> r, v, q, L;
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
	}
	check(md_upload_molecules(_ctx, (int64_t)id.size(), id.data(), comp.data(), r.data(), v.data(), q.data(),
							  L.data()),
		  "md_upload_molecules");
	_deviceStale = false;
	_hostStale = false;
}

void GpuLinkedCells::syncToHost() {
	if (!_ctx || !_hostStale) return;
	const size_t n = _ids.size();
	std::vector<double> r(3 * n), v(3 * n), q(4 * n), L(3 * n), F(3 * n), M(3 * n), Vi(3 * n);
	check(md_download_molecules(_ctx, (int64_t)n, nullptr, nullptr, r.data(), v.data(), q.data(), L.data(),
								F.data(), M.data(), Vi.data()),
		  "md_download_molecules");
	for (auto m = LinkedCells::iterator(ParticleIterator::ONLY_INNER_AND_BOUNDARY); m.isValid(); ++m) {
		const size_t k = _slot.at(m->getID());
		for (int d = 0; d < 3; ++d) {
			m->setr(d, r[3 * k + d]);
			m->setv(d, v[3 * k + d]);
			m->setD(d, L[3 * k + d]);
		}
		m->setq(Quaternion(q[4 * k], q[4 * k + 1], q[4 * k + 2], q[4 * k + 3]));
		m->setF(&F[3 * k]);
		m->setM(&M[3 * k]);
		m->setVi(&Vi[3 * k]);
	}
	_hostStale = false;
	LinkedCells::update();  // positions moved: re-bin the mirror
	_deviceStale = true;    // the caller may now edit molecules through the iterator
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
	syncToHost();
	return LinkedCells::iterator(t);
}

RegionParticleIterator GpuLinkedCells::regionIterator(const double startCorner[3], const double endCorner[3],
													  ParticleIterator::Type t) {
	syncToHost();
	return LinkedCells::regionIterator(startCorner, endCorner, t);
}

unsigned long GpuLinkedCells::getNumberOfParticles(ParticleIterator::Type t) {
	if (_ctx && !_deviceStale && t != ParticleIterator::ALL_CELLS) return _ids.size();
	return LinkedCells::getNumberOfParticles(t);
}
