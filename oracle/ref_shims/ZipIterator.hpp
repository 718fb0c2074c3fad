// Minimal stand-in for the un-vendored ZipIterator submodule of the reference
// (dpellegr/ZipIterator, pinned commit not mounted).  The reference's sources include
// <ZipIterator.hpp> only for `Zip(a, b, ...)` in a range-for with a structured binding
// (core/Simulation.cpp:733 over two containers; core/observables/Histogram.tpp:13-100
// and HistogramBuilder.tpp:86 over two or three).  This header is written for the oracle
// build and supports exactly that use: iterating equally long containers in lockstep,
// yielding a tuple of references.
#pragma once
#include <cstddef>
#include <iterator>
#include <tuple>
#include <utility>

namespace rpo_zip_shim {
template <typename... C>
class ZipRange {
    std::tuple<C &...> cs;

public:
    using Iters = std::tuple<decltype(std::begin(std::declval<C &>()))...>;
    class iterator {
        Iters its;

    public:
        explicit iterator(Iters its_) : its{its_} {}
        auto operator*() const {
            return std::apply([](auto &...i) { return std::tuple<decltype(*i)...>(*i...); }, its);
        }
        iterator &operator++() {
            std::apply([](auto &...i) { (++i, ...); }, its);
            return *this;
        }
        bool operator!=(const iterator &o) const { return std::get<0>(its) != std::get<0>(o.its); }
        bool operator==(const iterator &o) const { return std::get<0>(its) == std::get<0>(o.its); }
    };
    explicit ZipRange(C &...c) : cs{c...} {}
    iterator begin() const {
        return iterator(std::apply([](auto &...c) { return Iters(std::begin(c)...); }, cs));
    }
    iterator end() const {
        return iterator(std::apply([](auto &...c) { return Iters(std::end(c)...); }, cs));
    }
};
}  // namespace rpo_zip_shim

template <typename... C>
rpo_zip_shim::ZipRange<C...> Zip(C &...c) { return rpo_zip_shim::ZipRange<C...>(c...); }
