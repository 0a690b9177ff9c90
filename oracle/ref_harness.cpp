// Test-infrastructure-only pybind11 module over the reference C++ headers,
// compiled where they lie (cpp_ext/ of vbharadwaj-bk/fast_tensor_leverage)
// by oracle/Makefile.  Nothing here is shipped or timed as the product.
//
// The reference's own bindings (cpp_ext/als_module.cpp:64-68) always pass
// random_draws=nullptr, so its samples cannot be reproduced.  This module
// adds what the parity tests need:
//   * RefSampler.draw(j, samples, draws): EfficientKRPSampler::KRPDrawSamples
//     with injected uniforms (efficient_krp_sampler.hpp:209-268, layout 2N x J:
//     eigen draws of mode k at k*J, Gram draws at N*J + k*J);
//   * read-back of h, weights, the M workspace and every tree's node Grams;
//   * RefPartitionTree: the standalone tree (partition_tree.cpp:4-40);
//   * InjectedALS: ALS whose sampler consumes a caller-provided uniform block
//     (ALS::sampler is a public unique_ptr, als.hpp:25; KRPDrawSamples is
//     virtual, sampler.hpp:69).
#include <iostream>
#include <string>
#include <vector>
#include "common.h"
#include "cblas.h"
#include "lapacke.h"
#include "hashing.hpp"
#include "sampler.hpp"
#include "tensor.hpp"
#include "sparse_tensor.hpp"
#include "low_rank_tensor.hpp"
#include "dense_tensor.hpp"
#include "uniform_sampler.hpp"
#include "larsen_kolda_sampler.hpp"
#include "larsen_kolda_hybrid.hpp"
#include "efficient_krp_sampler.hpp"
#include "als.hpp"

#include <pybind11/pybind11.h>
#include <pybind11/numpy.h>

namespace py = pybind11;

class InjectedKRPSampler : public EfficientKRPSampler {
public:
    std::vector<double> draws;  // 2N x J when non-empty
    InjectedKRPSampler(uint64_t J, uint64_t R, vector<Buffer<double>> &U)
        : EfficientKRPSampler(J, R, U) {}

    void KRPDrawSamples(uint32_t j, Buffer<uint64_t> &samples,
                        Buffer<double> *random_draws) override {
        if (random_draws == nullptr && !draws.empty()) {
            Buffer<double> view({(uint64_t)draws.size()}, draws.data());
            EfficientKRPSampler::KRPDrawSamples(j, samples, &view);
        } else {
            EfficientKRPSampler::KRPDrawSamples(j, samples, random_draws);
        }
    }
};

static void copy_out(const double *src, size_t n, py::array_t<double> out) {
    auto info = out.request();
    if ((size_t)info.size < n) throw std::runtime_error("output buffer too small");
    std::copy(src, src + n, static_cast<double *>(info.ptr));
}

static void set_draws_from(std::vector<double> &dst, py::array_t<double> d) {
    auto info = d.request();
    const double *p = static_cast<const double *>(info.ptr);
    dst.assign(p, p + info.size);
}

class RefSampler {
public:
    unique_ptr<NPBufferList<double>> U_bufs;
    unique_ptr<InjectedKRPSampler> s;
    RefSampler(py::list U, int64_t J, int64_t R)
        : U_bufs(new NPBufferList<double>(U)) {
        s.reset(new InjectedKRPSampler(J, R, U_bufs->buffers));
    }
    void draw(uint32_t j, py::array_t<uint64_t> samples_py, py::array_t<double> draws_py) {
        Buffer<uint64_t> samples(samples_py);
        set_draws_from(s->draws, draws_py);
        s->KRPDrawSamples(j, samples, nullptr);
    }
    void get_h(py::array_t<double> out) { copy_out(s->h(), s->J * s->R, out); }
    void get_weights(py::array_t<double> out) { copy_out(s->weights(), s->J, out); }
    void get_M(py::array_t<double> out) { copy_out(s->M(), (s->N + 2) * s->R2, out); }
    void get_lambda(py::array_t<double> out) { copy_out(s->lambda(), (s->N + 1) * s->R, out); }
    void get_gram_G(int k, py::array_t<double> out) {
        auto *t = s->gram_trees[k];
        copy_out(t->G(), (size_t)t->node_count * t->R2, out);
    }
    void get_eigen_G(int k, py::array_t<double> out) {
        auto *t = s->eigen_trees[k];
        copy_out(t->G(), (size_t)t->node_count * t->R2, out);
    }
    void update_sampler(uint64_t j) { s->update_sampler(j); }
};

class RefPartitionTree {
public:
    ScratchBuffer scratch;
    PartitionTree tree;
    RefPartitionTree(uint32_t n, uint32_t F, uint64_t J, uint64_t R)
        : scratch(F, J, R), tree(n, F, J, R, scratch) {}
    void build_tree(py::array_t<double> U) {
        Buffer<double> Ub(U);
        tree.build_tree(Ub);
    }
    void multiply_against_numpy_buffer(py::array_t<double> m) { tree.multiply_against_numpy_buffer(m); }
    void PTSample(py::array_t<double> U, py::array_t<double> h, py::array_t<double> sh,
                  py::array_t<uint64_t> samples, py::array_t<double> draws) {
        tree.PTSample(U, h, sh, samples, draws);
    }
    void get_G0(py::array_t<double> out) { tree.get_G0(out); }
    void get_G(py::array_t<double> out) { copy_out(tree.G(), (size_t)tree.node_count * tree.R2, out); }
    py::dict geometry() {
        py::dict d;
        d["leaf_count"] = tree.leaf_count;
        d["node_count"] = tree.node_count;
        d["lfill_level"] = tree.lfill_level;
        d["lfill_count"] = tree.lfill_count;
        d["total_levels"] = tree.total_levels;
        d["nodes_upto_lfill"] = tree.nodes_upto_lfill;
        d["nodes_before_lfill"] = tree.nodes_before_lfill;
        d["complete_level_offset"] = tree.complete_level_offset;
        return d;
    }
};

class InjectedALS {
public:
    ALS als;
    InjectedKRPSampler *inj = nullptr;
    InjectedALS(LowRankTensor &lr, Tensor &gt) : als(lr, gt) {}
    void initialize_ds_als(uint64_t J) {
        uint64_t N = als.cp_decomp.N;
        inj = new InjectedKRPSampler(J, als.cp_decomp.R, als.cp_decomp.U);
        als.sampler.reset(inj);
        als.samples.reset(new Buffer<uint64_t>({N, J}));
        als.samples_transpose.reset(new Buffer<uint64_t>({J, N}));
    }
    void set_draws(py::array_t<double> d) { set_draws_from(inj->draws, d); }
    void execute_ds_als_update(uint32_t j, bool renorm, bool update) {
        als.execute_ds_als_update(j, renorm, update);
    }
    void execute_exact_als_update(uint32_t j, bool renorm, bool update) {
        als.execute_exact_als_update(j, renorm, update);
    }
    void get_samples(py::array_t<uint64_t> out) {
        auto info = out.request();
        uint64_t n = als.cp_decomp.N * inj->J;
        std::copy((*als.samples)(), (*als.samples)(n), static_cast<uint64_t *>(info.ptr));
    }
    void get_h(py::array_t<double> out) { copy_out(inj->h(), inj->J * inj->R, out); }
    void get_weights(py::array_t<double> out) { copy_out(inj->weights(), inj->J, out); }
};

static void set_blas_threads(int n) { scipy_openblas_set_num_threads(n); }

PYBIND11_MODULE(ftl_ref, m) {
    m.def("set_blas_threads", &set_blas_threads);
    m.def("set_omp_threads", [](int n) { omp_set_num_threads(n); });
    py::class_<Tensor>(m, "Tensor", py::module_local())
        .def("execute_downsampled_mttkrp_py", &Tensor::execute_downsampled_mttkrp_py)
        .def("compute_residual_normsq", &Tensor::compute_residual_normsq_py)
        .def("get_normsq", &Tensor::get_normsq);
    py::class_<BlackBoxTensor, Tensor>(m, "BlackBoxTensor", py::module_local());
    py::class_<LowRankTensor, BlackBoxTensor>(m, "LowRankTensor", py::module_local())
        .def(py::init<uint64_t, uint64_t, py::list>())
        .def(py::init<uint64_t, py::list>())
        .def("get_sigma", &LowRankTensor::get_sigma_py)
        .def("set_sigma", &LowRankTensor::set_sigma_py)
        .def("renormalize_columns", &LowRankTensor::renormalize_columns)
        .def("materialize_rhs", &LowRankTensor::materialize_rhs_py)
        .def("evaluate_indices", &LowRankTensor::evaluate_indices_py);
    py::class_<DenseTensor<double>, BlackBoxTensor>(m, "DenseTensor", py::module_local())
        .def(py::init<py::array_t<double>, uint64_t>());
    py::class_<SparseTensor, Tensor>(m, "SparseTensor", py::module_local())
        .def(py::init<py::array_t<uint32_t>, py::array_t<double>, std::string>())
        .def("execute_rrf", &SparseTensor::execute_rrf);
    py::class_<InjectedALS>(m, "InjectedALS", py::module_local())
        .def(py::init<LowRankTensor &, Tensor &>(), py::keep_alive<1, 2>(), py::keep_alive<1, 3>())
        .def("initialize_ds_als", &InjectedALS::initialize_ds_als)
        .def("set_draws", &InjectedALS::set_draws)
        .def("execute_ds_als_update", &InjectedALS::execute_ds_als_update)
        .def("execute_exact_als_update", &InjectedALS::execute_exact_als_update)
        .def("get_samples", &InjectedALS::get_samples)
        .def("get_h", &InjectedALS::get_h)
        .def("get_weights", &InjectedALS::get_weights);
    py::class_<RefSampler>(m, "RefSampler", py::module_local())
        .def(py::init<py::list, int64_t, int64_t>())
        .def("draw", &RefSampler::draw)
        .def("get_h", &RefSampler::get_h)
        .def("get_weights", &RefSampler::get_weights)
        .def("get_M", &RefSampler::get_M)
        .def("get_lambda", &RefSampler::get_lambda)
        .def("get_gram_G", &RefSampler::get_gram_G)
        .def("get_eigen_G", &RefSampler::get_eigen_G)
        .def("update_sampler", &RefSampler::update_sampler);
    py::class_<RefPartitionTree>(m, "RefPartitionTree", py::module_local())
        .def(py::init<uint32_t, uint32_t, uint64_t, uint64_t>())
        .def("build_tree", &RefPartitionTree::build_tree)
        .def("multiply_against_numpy_buffer", &RefPartitionTree::multiply_against_numpy_buffer)
        .def("PTSample", &RefPartitionTree::PTSample)
        .def("get_G0", &RefPartitionTree::get_G0)
        .def("get_G", &RefPartitionTree::get_G)
        .def("geometry", &RefPartitionTree::geometry);
}
