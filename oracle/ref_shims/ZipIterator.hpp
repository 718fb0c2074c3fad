// Minimal stand-in for the un-vendored ZipIterator submodule of the reference
// (dpellegr/ZipIterator, pinned commit not mounted).  The reference's hot-path
// sources include <ZipIterator.hpp> only for `Zip(a, b)` in a range-for with a
// structured binding (core/Simulation.cpp:733, move statistics).  This header is
// written for the oracle build and supports exactly that use: iterating two
// equally long containers in lockstep and yielding a pair of references.
#pragma once
#include <cstddef>
#include <utility>
#include <iterator>

namespace rpo_zip_shim {
template <typename A, typename B>
class ZipRange {
    A &a;
    B &b;
public:
    using IA = decltype(std::begin(std::declval<A &>()));
    using IB = decltype(std::begin(std::declval<B &>()));
    class iterator {
        IA ia;
        IB ib;
    public:
        iterator(IA ia_, IB ib_) : ia{ia_}, ib{ib_} {}
        auto operator*() const { return std::pair<decltype(*ia), decltype(*ib)>(*ia, *ib); }
        iterator &operator++() { ++ia; ++ib; return *this; }
        bool operator!=(const iterator &o) const { return ia != o.ia; }
        bool operator==(const iterator &o) const { return ia == o.ia; }
    };
    ZipRange(A &a_, B &b_) : a{a_}, b{b_} {}
    iterator begin() const { return iterator(std::begin(a), std::begin(b)); }
    iterator end() const { return iterator(std::end(a), std::end(b)); }
};
}  // namespace rpo_zip_shim

template <typename A, typename B>
rpo_zip_shim::ZipRange<A, B> Zip(A &a, B &b) { return rpo_zip_shim::ZipRange<A, B>(a, b); }
