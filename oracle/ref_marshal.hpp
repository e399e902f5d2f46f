// ORACLE — test infrastructure only (see oracle_common.hpp).
//
// Marshalling between flat double buffers and the reference's
// numeric::tuple_t / nd::shared_array types, shared by the reference
// harnesses (ref_harness.cpp, ref_harness_v2.cpp). Include after the
// reference headers that define the tuple and array types.
#pragma once
#include <array>
#include <cstddef>
#include <utility>

namespace {

template<typename Tuple, std::size_t... I>
void load_tuple(Tuple& t, const double* src, std::index_sequence<I...>)
{
    ((std::get<I>(t.impl).value = src[I]), ...);
}

template<typename Tuple, std::size_t... I>
void store_tuple(const Tuple& t, double* dst, std::index_sequence<I...>)
{
    ((dst[I] = std::get<I>(t.impl).value), ...);
}

template<typename Tuple>
constexpr std::size_t tuple_size_v = std::tuple_size_v<decltype(Tuple().impl)>;

template<typename Tuple>
Tuple to_tuple(const double* src)
{
    Tuple t;
    load_tuple(t, src, std::make_index_sequence<tuple_size_v<Tuple>>());
    return t;
}

template<typename Tuple>
void from_tuple(const Tuple& t, double* dst)
{
    store_tuple(t, dst, std::make_index_sequence<tuple_size_v<Tuple>>());
}

template<typename Tuple>
nd::shared_array<Tuple, 2> make_array2(const double* data, std::size_t n0, std::size_t n1)
{
    constexpr auto K = tuple_size_v<Tuple>;
    auto a = nd::make_unique_array<Tuple, 2>(nd::uivec(n0, n1));
    for (std::size_t i = 0; i < n0; ++i)
        for (std::size_t j = 0; j < n1; ++j)
            a(i, j) = to_tuple<Tuple>(data + (i * n1 + j) * K);
    return nd::make_shared_array(std::move(a));
}

template<typename Tuple>
void read_array2(const nd::shared_array<Tuple, 2>& a, double* out)
{
    constexpr auto K = tuple_size_v<Tuple>;
    auto n0 = shape(a, 0), n1 = shape(a, 1);
    for (std::size_t i = 0; i < n0; ++i)
        for (std::size_t j = 0; j < n1; ++j)
            from_tuple(a(i, j), out + (i * n1 + j) * K);
}

template<typename Tuple>
nd::shared_array<Tuple, 3> make_array3(const double* data, std::size_t n0, std::size_t n1, std::size_t n2)
{
    constexpr auto K = tuple_size_v<Tuple>;
    auto a = nd::make_unique_array<Tuple, 3>(nd::uivec(n0, n1, n2));
    for (std::size_t i = 0; i < n0; ++i)
        for (std::size_t j = 0; j < n1; ++j)
            for (std::size_t k = 0; k < n2; ++k)
                a(i, j, k) = to_tuple<Tuple>(data + ((i * n1 + j) * n2 + k) * K);
    return nd::make_shared_array(std::move(a));
}

template<typename Array>
void read_array3(const Array& a, double* out)
{
    using Tuple = typename Array::value_type;
    constexpr auto K = tuple_size_v<Tuple>;
    auto n0 = shape(a, 0), n1 = shape(a, 1), n2 = shape(a, 2);
    for (std::size_t i = 0; i < n0; ++i)
        for (std::size_t j = 0; j < n1; ++j)
            for (std::size_t k = 0; k < n2; ++k)
                from_tuple(a(i, j, k), out + ((i * n1 + j) * n2 + k) * K);
}

template<typename Q>
nd::shared_array<Q, 3> make_scalar3(const double* data, std::size_t n0, std::size_t n1, std::size_t n2)
{
    auto a = nd::make_unique_array<Q, 3>(nd::uivec(n0, n1, n2));
    for (std::size_t i = 0; i < n0; ++i)
        for (std::size_t j = 0; j < n1; ++j)
            for (std::size_t k = 0; k < n2; ++k)
                a(i, j, k) = Q(data[(i * n1 + j) * n2 + k]);
    return nd::make_shared_array(std::move(a));
}

template<typename Array>
void read_scalar3(const Array& a, double* out)
{
    auto n0 = shape(a, 0), n1 = shape(a, 1), n2 = shape(a, 2);
    for (std::size_t i = 0; i < n0; ++i)
        for (std::size_t j = 0; j < n1; ++j)
            for (std::size_t k = 0; k < n2; ++k)
                out[(i * n1 + j) * n2 + k] = a(i, j, k).value;
}

// the three face (or edge) arrays of a block whose cell shape is (n0, n1, n2),
// each longer by `grow` along its own axis and by `side` on the other two
std::array<nd::uivec_t<3>, 3> staggered_shapes(std::size_t n0, std::size_t n1, std::size_t n2, long grow, long side)
{
    auto g = [] (std::size_t n, long d) { return std::size_t(long(n) + d); };
    return {nd::uivec(g(n0, grow), g(n1, side), g(n2, side)), nd::uivec(g(n0, side), g(n1, grow), g(n2, side)),
            nd::uivec(g(n0, side), g(n1, side), g(n2, grow))};
}

} // namespace
