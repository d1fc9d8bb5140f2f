# SwalbeGB300.jl -- Julia binding of libswalbe_gb300.so for Swalbe.jl.
#
# Makes `Sys(sysc, "GB300"; T)` return a `GB300State <: Swalbe.LBM_state_2D`
# whose `time_loop` methods run the fused GB300 step through the C ABI
# (include/swalbe_gb300.h), one ccall per loop instead of ~70 broadcasts per
# iteration (src/simulate.jl:6-96).  Host arrays are the state's mirrors:
# `height`, `velx`, `vely` are uploaded at the start of each `time_loop` and
# refreshed at its end, so code that writes `state.height .= ...` before the
# loop and reads `state.height` after it works unchanged.
#
# The library path comes from ENV["SWALBE_GB300_LIB"], else the in-tree build
# (../lib/libswalbe_gb300.so).
module SwalbeGB300

import Swalbe

const libswb = get(ENV, "SWALBE_GB300_LIB",
                   joinpath(@__DIR__, "..", "lib", "libswalbe_gb300.so"))

# status codes and modes (include/swalbe_gb300.h)
const SWB_OK = Cint(0)
const SWB_ERR_NAN = Cint(-4)
const PRECISION = Dict(Float64 => Cint(0), Float32 => Cint(1), Float16 => Cint(2))
const SWB_PLAIN64 = Cint(3)
const FIELD_HEIGHT, FIELD_VELX, FIELD_VELY, FIELD_PRESSURE = Cint(0), Cint(1), Cint(2), Cint(3)
const MEAS_MASS, MEAS_WETTED, MEAS_MAXMIN, MEAS_AREA = Cint(1), Cint(2), Cint(4), Cint(8)

# swb_params: the same field order and C types
struct SwbParams
    Lx::Int32; Ly::Int32; Tmax::Int32; tdump::Int32
    tau::Float64; cs::Float64; mu::Float64
    delta::Float64; kbt::Float64
    gamma::Float64
    n::Int32; m::Int32
    hmin::Float64; hcrit::Float64
    theta::Float64; g::Float64
end

struct SwbMeasure
    t::Int64; mass::Float64; wetted::Int64
    hmax::Float64; hmin::Float64; area::Float64; energy::Float64
end

function SwbParams(sys::Swalbe.SysConst)
    p = sys.param
    SwbParams(sys.Lx, sys.Ly, p.Tmax, p.tdump, p.τ, p.cₛ, p.μ, p.δ, p.kbt, p.γ, p.n, p.m,
              p.hmin, p.hcrit, p.θ, p.g)
end

struct SwbError <: Exception
    status::Cint
    msg::String
end
Base.showerror(io::IO, e::SwbError) = print(io, "swalbe_gb300 error ", e.status, ": ", e.msg)

function check(st::Cint, h::Ptr{Cvoid})
    st == SWB_OK && return nothing
    msg = unsafe_string(ccall((:swb_last_error, libswb), Cstring, (Ptr{Cvoid},), h))
    throw(SwbError(st, msg))
end

"""
    GB300State(sys; T = Float64, plain = false)

A lattice on the GPU.  `T` = Float64 (the reference's arithmetic, bit for
bit), Float32 (FP32) or Float16 (FP32 arithmetic, FP16 populations).
`plain = true` selects one kernel per reference op (Float64 only), for
scripts that call `filmpressure!`, `h∇p!`, ... themselves.
"""
mutable struct GB300State <: Swalbe.LBM_state_2D
    handle::Ptr{Cvoid}
    sys::Swalbe.SysConst
    height::Matrix{Float64}
    velx::Matrix{Float64}
    vely::Matrix{Float64}
    pressure::Matrix{Float64}
end

function GB300State(sys::Swalbe.SysConst; T = Float64, plain = false)
    prec = plain ? SWB_PLAIN64 : PRECISION[T]
    ref = Ref{Ptr{Cvoid}}(C_NULL)
    p = Ref(SwbParams(sys))
    check(ccall((:swb_create, libswb), Cint, (Ref{SwbParams}, Cint, Ref{Ptr{Cvoid}}), p, prec, ref),
          C_NULL)
    s = GB300State(ref[], sys, ones(sys.Lx, sys.Ly), zeros(sys.Lx, sys.Ly),
                   zeros(sys.Lx, sys.Ly), zeros(sys.Lx, sys.Ly))
    finalizer(s) do x
        x.handle == C_NULL || ccall((:swb_destroy, libswb), Cint, (Ptr{Cvoid},), x.handle)
        x.handle = C_NULL
    end
    return s
end

set_field!(s::GB300State, f::Cint, a::Matrix{Float64}) =
    check(ccall((:swb_set_field, libswb), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}), s.handle, f, a),
          s.handle)
get_field!(a::Matrix{Float64}, s::GB300State, f::Cint) =
    check(ccall((:swb_get_field, libswb), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}), s.handle, f, a),
          s.handle)

function upload!(s::GB300State)
    set_field!(s, FIELD_HEIGHT, s.height)
    set_field!(s, FIELD_VELX, s.velx)
    set_field!(s, FIELD_VELY, s.vely)
end

function download!(s::GB300State)
    get_field!(s.height, s, FIELD_HEIGHT)
    get_field!(s.velx, s, FIELD_VELX)
    get_field!(s.vely, s, FIELD_VELY)
    return s
end

set_theta!(s::GB300State, θ::Number) =
    check(ccall((:swb_set_theta, libswb), Cint, (Ptr{Cvoid}, Cdouble), s.handle, θ), s.handle)
set_theta!(s::GB300State, θ::AbstractMatrix) =
    check(ccall((:swb_set_theta_field, libswb), Cint, (Ptr{Cvoid}, Ptr{Float64}), s.handle,
                Matrix{Float64}(θ)), s.handle)
set_measures!(s::GB300State, mask, hthresh = 0.055) =
    check(ccall((:swb_set_measures, libswb), Cint, (Ptr{Cvoid}, Cint, Cdouble), s.handle, mask,
                hthresh), s.handle)

function step!(s::GB300State, n::Integer)
    check(ccall((:swb_step, libswb), Cint, (Ptr{Cvoid}, Int64), s.handle, n), s.handle)
    check(ccall((:swb_sync, libswb), Cint, (Ptr{Cvoid},), s.handle), s.handle)
end

function measures(s::GB300State, n::Integer)
    out = Vector{SwbMeasure}(undef, n)
    cnt = Ref{Int64}(0)
    check(ccall((:swb_get_measures, libswb), Cint,
                (Ptr{Cvoid}, Ptr{SwbMeasure}, Int64, Ref{Int64}), s.handle, out, n, cnt), s.handle)
    return resize!(out, cnt[])
end

function run!(sys, s::GB300State; verbose = false)
    Tmax, tdump = sys.param.Tmax, sys.param.tdump
    upload!(s)
    done = 0
    while done < Tmax
        n = verbose ? min(tdump - done % tdump, Tmax - done) : Tmax - done
        step!(s, n)
        done += n
        if verbose && done % tdump == 0
            get_field!(s.height, s, FIELD_HEIGHT)
            println("Time step $done mass is $(round(sum(s.height), digits=3))")
        end
    end
    return download!(s)
end

# time_loop(sys, state) and time_loop(sys, state, θ) (src/simulate.jl:6-45)
function Swalbe.time_loop(sys::Swalbe.SysConst, s::GB300State; verbose = false)
    set_measures!(s, 0)
    run!(sys, s; verbose)
end
function Swalbe.time_loop(sys::Swalbe.SysConst, s::GB300State, θ; verbose = false)
    set_theta!(s, θ)
    set_measures!(s, 0)
    run!(sys, s; verbose)
end
# time_loop(sys, state, Δh) (src/simulate.jl:47-66): max - min every iteration
function Swalbe.time_loop(sys::Swalbe.SysConst, s::GB300State, Δh::Vector; verbose = false)
    set_measures!(s, MEAS_MAXMIN)
    run!(sys, s; verbose)
    append!(Δh, (m.hmax - m.hmin for m in measures(s, sys.param.Tmax)))
    return s
end
# time_loop(sys, state, f, measure) (src/simulate.jl:68-96): wetted! is fused;
# any other callback needs the forces on the host every iteration
function Swalbe.time_loop(sys::Swalbe.SysConst, s::GB300State, f::Function, measure::Vector;
                          verbose = false)
    f === Swalbe.wetted! || throw(ArgumentError(
        "GB300State fuses wetted! only; run other per-iteration callbacks on a CPU State"))
    set_measures!(s, MEAS_WETTED)
    run!(sys, s; verbose)
    append!(measure, (m.wetted for m in measures(s, sys.param.Tmax)))
    return s, measure
end

# The per-op methods on a plain state (one kernel per reference op).
for (jl, c) in ((:filmpressure!, :swb_op_filmpressure), (:slippage!, :swb_op_slippage),
                (:equilibrium!, :swb_op_equilibrium), (:BGKandStream!, :swb_op_bgk_stream))
    @eval function Swalbe.$jl(s::GB300State, sys::Swalbe.SysConst)
        check(ccall(($(QuoteNode(c)), libswb), Cint, (Ptr{Cvoid},), s.handle), s.handle)
    end
end
Swalbe.h∇p!(s::GB300State) =
    check(ccall((:swb_op_hgradp, libswb), Cint, (Ptr{Cvoid},), s.handle), s.handle)
Swalbe.moments!(s::GB300State) =
    check(ccall((:swb_op_moments, libswb), Cint, (Ptr{Cvoid},), s.handle), s.handle)

end  # module
