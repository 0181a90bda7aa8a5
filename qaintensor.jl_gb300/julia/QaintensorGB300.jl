"""
    QaintensorGB300

ccall bindings of libqaintensor_gb300.so for Qaintensor.jl (the C ABI is
declared in include/qaintensor_gb300.h).  Julia arrays are column-major with
interleaved complex elements, exactly the layout the library takes, so no
conversion happens at the boundary; `GC.@preserve` keeps them alive across
each call.  Not exercised here: this image has no Julia.
"""
module QaintensorGB300

using LinearAlgebra
import Qaintensor: Tensor, MPS, contract_svd

const lib = get(ENV, "QAINTENSOR_GB300_LIB", joinpath(@__DIR__, "..", "libqaintensor_gb300.so"))

const QT_OK = Cint(0)
const QT_C64, QT_C128 = Cint(0), Cint(1)
const MODES = Dict(:plain => Cint(0), :chosen => Cint(1), :cusolver => Cint(2))

# the reference's own messages (src/svd.jl:9,16; src/mps.jl:195)
const MESSAGES = Dict(Cint(-1) => "Error must be positive",
                      Cint(-2) => "Dimensions of contraction legs do not match",
                      Cint(-9) => "Function doesn't support periodic boundary conditions for now")

struct QtConfig
    device::Cint; mode::Cint; cutoff::Cdouble; chi_max::Cint; oversample::Cint; power_iters::Cint
    renormalize::Cint; use_rank_model::Cint; max_sweeps::Cint; jacobi_tol::Cdouble; noise_floor::Cdouble
    seed::UInt64; tc_gemm::Cint; jacobi_kernel::Cint
end

struct QtUpdateStats
    rank::Cint; rank_cutoff::Cint; predicted_rank::Cint; sketch_size::Cint; fallback::Cint; sweeps::Cint
    discarded_weight::Cdouble; norm2::Cdouble; residual::Cdouble
end

mutable struct Engine
    h::Ptr{Cvoid}
end

function check(e::Engine, rc::Cint)
    rc == QT_OK && return
    haskey(MESSAGES, rc) && error(MESSAGES[rc])
    rc == Cint(-10) && throw(BoundsError())
    error(unsafe_string(ccall((:qt_last_error, lib), Cstring, (Ptr{Cvoid},), e.h)))
end

function Engine(; mode::Symbol=:plain, cutoff=0.0, chi_max=0, device=0, tc_gemm=true)
    cfg = Ref{QtConfig}()
    ccall((:qt_config_default, lib), Cint, (Ref{QtConfig},), cfg)
    c = cfg[]
    cfg[] = QtConfig(device, MODES[mode], cutoff, chi_max, c.oversample, c.power_iters, c.renormalize,
                     c.use_rank_model, c.max_sweeps, c.jacobi_tol, c.noise_floor, c.seed, Cint(tc_gemm),
                     c.jacobi_kernel)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    rc = ccall((:qt_create, lib), Cint, (Ref{Ptr{Cvoid}}, Ref{QtConfig}), h, cfg)
    rc == QT_OK || error("qt_create failed ($rc)")
    e = Engine(h[])
    finalizer(x -> ccall((:qt_destroy, lib), Cint, (Ptr{Cvoid},), x.h), e)
    return e
end

dtype(::Type{ComplexF64}) = QT_C128
dtype(::Type{ComplexF32}) = QT_C64

"""
    contract_svd(e::Engine, T1::Tensor, T2::Tensor, indx; er=0.0)

`contract_svd` of src/svd.jl:7-38 on the GPU: same legs, same two truncated
SVDs and tail rule, same output leg order.
"""
function contract_svd(e::Engine, T1::Tensor, T2::Tensor, indx::NTuple{2,Int}; er=0.0)
    er >= 0 || error("Error must be positive")
    T = promote_type(eltype(T1.data), eltype(T2.data), ComplexF32)
    a, b = convert(Array{T}, T1.data), convert(Array{T}, T2.data)
    i1, i2 = indx
    s1, s2 = size(a), size(b)
    newdim = [s1[1:i1-1]...; s1[i1+1:end]...; s2[1:i2-1]...; s2[i2+1:end]...]
    out = Array{T}(undef, newdim...)
    GC.@preserve a b out begin
        rc = ccall((:qt_contract_svd, lib), Cint,
                   (Ptr{Cvoid}, Cint, Cint, Ptr{Int64}, Ptr{Cvoid}, Cint, Ptr{Int64}, Ptr{Cvoid}, Cint, Cint, Cdouble, Ptr{Cvoid}),
                   e.h, dtype(T), ndims(a), collect(Int64, s1), a, ndims(b), collect(Int64, s2), b, i1, i2, er, out)
    end
    check(e, rc)
    return Tensor(out)
end

"""A device-resident copy of an MPS (sites (chiL, 2, chiR)); end tensors of
`MPS(psi)`/`ClosedMPS` ((2, chi) and (chi, 2)) are passed as they are: the
memory is identical to (1, 2, chi) and (chi, 2, 1)."""
mutable struct DeviceMPS
    e::Engine
    p::Ptr{Cvoid}
    T::DataType
end

function DeviceMPS(e::Engine, mps::MPS; T=ComplexF64)
    n = length(mps.tensors)
    dims = Int64[]
    datas = [convert(Array{T}, t.data) for t in mps.tensors]
    for (i, d) in enumerate(datas)
        s = size(d)
        if ndims(d) == 3
            append!(dims, s)
        elseif i == 1
            append!(dims, (1, s...))
        else
            append!(dims, (s..., 1))
        end
    end
    out = Ref{Ptr{Cvoid}}(C_NULL)
    ptrs = [pointer(d) for d in datas]
    GC.@preserve datas begin
        rc = ccall((:qt_mps_create, lib), Cint, (Ptr{Cvoid}, Cint, Ptr{Int64}, Ptr{Ptr{Cvoid}}, Cint, Ref{Ptr{Cvoid}}),
                   e.h, n, dims, ptrs, dtype(T), out)
    end
    check(e, rc)
    m = DeviceMPS(e, out[], T)
    finalizer(x -> ccall((:qt_mps_free, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), x.e.h, x.p), m)
    return m
end

"""
    apply_2q!(m::DeviceMPS, G::Matrix, i; cutoff=-1, chi_max=-1, mode=nothing)

Gate G (4x4, U on the input legs, wire i = fastest bit) on wires (i, i+1),
then the truncated-SVD split (U to the left, diag(S)V' to the right).
"""
function apply_2q!(m::DeviceMPS, G::AbstractMatrix, i::Integer; cutoff=-1.0, chi_max=-1, mode=nothing)
    g = convert(Matrix{ComplexF64}, G)
    st = Ref{QtUpdateStats}()
    md = mode === nothing ? Cint(-1) : MODES[mode]
    GC.@preserve g begin
        rc = ccall((:qt_apply_2q, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{ComplexF64}, Cdouble, Cint, Cint, Ref{QtUpdateStats}),
                   m.e.h, m.p, i - 1, g, cutoff, chi_max, md, st)
    end
    check(m.e, rc)
    return st[]
end

"""`switch!(mps, i)` of src/switch.jl on the device."""
function switch!(m::DeviceMPS, i::Integer)
    check(m.e, ccall((:qt_switch, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint), m.e.h, m.p, i - 1))
end

function site(m::DeviceMPS, i::Integer)
    d = Vector{Int64}(undef, 3)
    ccall((:qt_mps_site_dims, lib), Cint, (Ptr{Cvoid}, Cint, Ptr{Int64}), m.p, i - 1, d)
    out = Array{m.T}(undef, d...)
    check(m.e, ccall((:qt_mps_download, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cvoid}), m.e.h, m.p, i - 1, out))
    return out
end

function expect_z(m::DeviceMPS, i::Integer)
    r = Ref{Cdouble}()
    check(m.e, ccall((:qt_expect_z, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ref{Cdouble}), m.e.h, m.p, i - 1, r))
    return r[]
end

end # module
