// qpc_gb300_lgwz.hpp -- drop-in replacement for the reference's
// propagator_cn_hc_lgwz<dims_t> (spherical/propagator/cn_1e.hpp:549-619) that
// runs the time step on a GB300 through the C ABI of include/qpc_gb300.h.
//
// Header-only C++17, to be included by the reference's driver after
// <spherical/inventory.h> (it uses the reference's own integrator_radi,
// operator_sc, operator_hc, operator_rpow1 and coefficient types, so that the
// members callers touch -- prop.s and prop.h, binsrc/sphTDSE.cpp:771-776 and
// 427-428 -- keep their types).  Link with libqpc_gb300.so.
//
//   initialize(nthd, radi, angu, mass, potn, dt)   same arguments as the reference
//   propagate(coef, ez_ti, ez_tf)                  one step, coef on the host (copied in and out)
//   propagate(coef)                                one field-free step
//   run(coef, f, nt_field, nt_total)               the whole driver loop on the device:
//                                                  f[i] = f(t_i), i = 0..nt_field
// Errors from the engine are thrown as the reference's errn_t from
// initialize (as the reference's own initialize does) and reported through
// last_status() from the noexcept propagate overloads.
#pragma once
#include "qpc_gb300.h"
#include <vector>
#include <string>

namespace qpc_gb300 {

template <class dims_t>
struct propagator_cn_hc_lgwz {
	qpc::spherical::operator_sc<dims_t> s;
	qpc::spherical::operator_hc<dims_t> h;
	qpc::spherical::operator_rpow1<dims_t> r;
	qpc_lgwz* handle = nullptr;
	int status = QPC_OK;

	propagator_cn_hc_lgwz() = default;
	propagator_cn_hc_lgwz(const propagator_cn_hc_lgwz&) = delete;
	propagator_cn_hc_lgwz& operator=(const propagator_cn_hc_lgwz&) = delete;
	~propagator_cn_hc_lgwz() { qpc_lgwz_destroy(handle); }

	int last_status() const noexcept { return status; }

	template <class potn_t>
	void initialize(size_t /*nthd*/, const qpc::spherical::integrator_radi<dims_t>& radi,
		const qpc::spherical::integrator_angu<dims_t>& /*angu*/, double mass, const potn_t& potn, double dt)
	{
		s.initialize(radi);
		r.initialize(radi);
		h.initialize(radi, mass, potn);
		const size_t nrs = dims_t::n_rsub, nl = dims_t::n_lmax + 1;
		std::vector<double> S(s.sub(), s.sub() + nrs), R(r.data, r.data + nrs), H(nl * nrs);
		// entries past the last B-spline are zero in the engine's band convention
		for (size_t i = 0; i < dims_t::n_dims; ++i)
			for (size_t k = 0; k < dims_t::n_elem; ++k)
				if (i + k >= dims_t::n_dims) { S[i * dims_t::n_elem + k] = 0.0; R[i * dims_t::n_elem + k] = 0.0; }
		for (size_t l = 0; l < nl; ++l)
			for (size_t i = 0; i < nrs; ++i)
				H[l * nrs + i] = (i / dims_t::n_elem + i % dims_t::n_elem >= dims_t::n_dims) ? 0.0 : h[l][i];
		qpc_dims d{(int32_t)dims_t::n_dims, (int32_t)dims_t::n_diag, (int32_t)dims_t::l_dims, (int32_t)dims_t::m_dims,
			(int32_t)dims_t::m_init, 1};
		qpc_lgwz_destroy(handle);
		handle = nullptr;
		status = qpc_lgwz_create(&d, dt, S.data(), R.data(), H.data(), &handle);
		if (status != QPC_OK) throw qpc::spherical::errn_t(std::string("qpc_lgwz_create: ") + qpc_last_error());
	}

	void propagate(qpc::spherical::coefficient<dims_t>& coef, double ez_ti, double ez_tf) noexcept
	{
		if ((status = qpc_lgwz_put(handle, (const double*)coef.data))) return;
		if ((status = qpc_lgwz_propagate(handle, &ez_ti, &ez_tf))) return;
		status = qpc_lgwz_get(handle, (double*)coef.data);
	}

	void propagate(qpc::spherical::coefficient<dims_t>& coef) noexcept
	{
		if ((status = qpc_lgwz_put(handle, (const double*)coef.data))) return;
		if ((status = qpc_lgwz_propagate_free(handle))) return;
		status = qpc_lgwz_get(handle, (double*)coef.data);
	}

	// the driver loop of binsrc/sphTDSE.cpp:786-831 without per-step observation
	int run(qpc::spherical::coefficient<dims_t>& coef, const double* f, int64_t nt_field, int64_t nt_total) noexcept
	{
		if ((status = qpc_lgwz_put(handle, (const double*)coef.data))) return status;
		if ((status = qpc_lgwz_run(handle, f, nt_field + 1, &nt_field, &nt_total))) return status;
		return status = qpc_lgwz_get(handle, (double*)coef.data);
	}
};

} // namespace qpc_gb300
