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
const SWB_ERR_ARG = Cint(-1)
const SWB_ERR_NAN = Cint(-4)
const SWB_ERR_NOT_FOUND = Cint(-7)
const SWB_ERR_BUSY = Cint(-8)
const PRECISION = Dict(Float64 => Cint(0), Float32 => Cint(1), Float16 => Cint(2))
const SWB_PLAIN64 = Cint(3)
const FIELD_HEIGHT, FIELD_VELX, FIELD_VELY, FIELD_PRESSURE = Cint(0), Cint(1), Cint(2), Cint(3)
const FIELD_FOUT, FIELD_FX, FIELD_FY = Cint(4), Cint(6), Cint(7)
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
    plain::Bool
    height::Matrix{Float64}
    velx::Matrix{Float64}
    vely::Matrix{Float64}
    pressure::Matrix{Float64}
    Fx::Matrix{Float64}  # plain states: the forces a callback sees and may change
    Fy::Matrix{Float64}
end

function GB300State(sys::Swalbe.SysConst; T = Float64, plain = false)
    prec = plain ? SWB_PLAIN64 : PRECISION[T]
    ref = Ref{Ptr{Cvoid}}(C_NULL)
    p = Ref(SwbParams(sys))
    check(ccall((:swb_create, libswb), Cint, (Ref{SwbParams}, Cint, Ref{Ptr{Cvoid}}), p, prec, ref),
          C_NULL)
    z() = zeros(sys.Lx, sys.Ly)
    s = GB300State(ref[], sys, plain, ones(sys.Lx, sys.Ly), z(), z(), z(), z(), z())
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

# The device ring holds SWB_RECORD_CAPACITY per-step records: loops step in
# chunks no longer than that and drain after each (the reference pushes
# Δh and wetted! every step, src/simulate.jl:56, src/measures.jl:13-17).
const RECORD_CAPACITY = 65536

measures_dropped(s::GB300State) = (n = Ref{Int64}(0);
    check(ccall((:swb_measures_dropped, libswb), Cint, (Ptr{Cvoid}, Ref{Int64}), s.handle, n),
          s.handle); n[])

# Tmax iterations; `drain(records)` receives each chunk's per-step records.
function run!(sys, s::GB300State; verbose = false, drain = nothing)
    Tmax, tdump = sys.param.Tmax, sys.param.tdump
    upload!(s)
    drain === nothing || measures(s, RECORD_CAPACITY)  # records of earlier calls
    dropped0 = measures_dropped(s)
    done = 0
    while done < Tmax
        n = min(Tmax - done, RECORD_CAPACITY)
        verbose && (n = min(n, tdump - done % tdump))
        step!(s, n)
        done += n
        drain === nothing || drain(measures(s, n))
        if verbose && done % tdump == 0
            get_field!(s.height, s, FIELD_HEIGHT)
            println("Time step $done mass is $(round(sum(s.height), digits=3))")
        end
    end
    measures_dropped(s) == dropped0 ||
        throw(SwbError(Cint(-1), "per-step records were overwritten before they were read"))
    return download!(s)
end

set_inclination!(s::GB300State, α; t = 1000, tstart = 0, tsmooth = 1, loop_time = false) =
    check(ccall((:swb_set_inclination, libswb), Cint,
                (Ptr{Cvoid}, Cdouble, Cdouble, Cint, Int64, Int64, Int64), s.handle, α[1], α[2],
                loop_time, t, tstart, tsmooth), s.handle)

"""
    set_theta_wave!(s, θ₀, Δθ, v)

Moving wettability θ(x, t) = θ₀ + Δθ sinpi(2(x - v t)/Lx), evaluated in the
kernels (scripts/Moving_wettability_structs.jl:183-186).
"""
set_theta_wave!(s::GB300State, θ0, dθ, v) =
    check(ccall((:swb_set_theta_wave, libswb), Cint, (Ptr{Cvoid}, Cdouble, Cdouble, Cdouble),
                s.handle, θ0, dθ, v), s.handle)

"""
    move_substrate!(s, tmove; direction = "diagonal")

move_substrate! of scripts/Moving_wettability_structs.jl:139-152 on the
device: the θ field set last moves one cell along `direction` after every
`tmove` iterations from now (no copy; tmove = 0 stops it).
"""
function move_substrate!(s::GB300State, tmove; direction = "diagonal")
    dx, dy = Dict("diagonal" => (1, 1), "x" => (1, 0), "y" => (0, 1))[direction]
    check(ccall((:swb_set_substrate_motion, libswb), Cint, (Ptr{Cvoid}, Int64, Cint, Cint),
                s.handle, tmove, dx, dy), s.handle)
end

"""
    set_snapshots!(s, dumping; capacity = 64), snapshots(s)

snapshot!(fluid, height, t; dumping) (src/measures.jl:99-105) on the device:
the height after every `dumping`-th iteration goes into a device ring;
`snapshots` returns the ones taken since the last call as the rows of a
matrix (the reference's `vec(h)` rows) and their iterations.
"""
set_snapshots!(s::GB300State, dumping; capacity = 64) =
    check(ccall((:swb_set_snapshots, libswb), Cint, (Ptr{Cvoid}, Int64, Int64), s.handle,
                dumping, capacity), s.handle)
function snapshots(s::GB300State; cap = 4096)
    N = s.sys.Lx * s.sys.Ly
    buf = Vector{Float64}(undef, cap * N)
    times = Vector{Int64}(undef, cap)
    cnt = Ref{Int64}(0)
    check(ccall((:swb_get_snapshots, libswb), Cint,
                (Ptr{Cvoid}, Ptr{Float64}, Int64, Ref{Int64}, Ptr{Int64}), s.handle, buf, cap, cnt,
                times), s.handle)
    n = cnt[]
    return permutedims(reshape(buf[1:n*N], N, n)), times[1:n]
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
    run!(sys, s; verbose, drain = recs -> append!(Δh, (m.hmax - m.hmin for m in recs)))
    return s
end

# One iteration of the reference's op sequence on a plain state with the
# callback after the forces (src/simulate.jl:84-94); the callback sees the
# state's host mirrors of height, velx, vely, Fx and Fy, and its changes to
# Fx and Fy reach the device.
function callback_iteration!(sys, s::GB300State, f, measure)
    for op in (:swb_op_filmpressure, :swb_op_hgradp, :swb_op_slippage, :swb_op_force_sum)
        check(ccall((op, libswb), Cint, (Ptr{Cvoid},), s.handle), s.handle)
    end
    download!(s)
    get_field!(s.Fx, s, FIELD_FX)
    get_field!(s.Fy, s, FIELD_FY)
    f(measure, s)
    set_field!(s, FIELD_FX, s.Fx)
    set_field!(s, FIELD_FY, s.Fy)
    for op in (:swb_op_equilibrium, :swb_op_bgk_stream, :swb_op_moments)
        check(ccall((op, libswb), Cint, (Ptr{Cvoid},), s.handle), s.handle)
    end
end

# time_loop(sys, state, f, measure) (src/simulate.jl:68-96): wetted! is a
# fused measure and inclination! a fused force (with the callback's default
# t = 1000); any other callback runs between the ops of the per-op Float64
# path, on the state itself when it is plain, else on a plain twin that
# starts from the state's populations and fields and hands them back.
function Swalbe.time_loop(sys::Swalbe.SysConst, s::GB300State, f::Function, measure::Vector;
                          verbose = false)
    if f === Swalbe.wetted!
        set_measures!(s, MEAS_WETTED)
        run!(sys, s; verbose, drain = recs -> append!(measure, (m.wetted for m in recs)))
    elseif f === Swalbe.inclination!
        set_measures!(s, 0)
        set_inclination!(s, measure)
        run!(sys, s; verbose)
        set_inclination!(s, (0.0, 0.0))
    elseif s.plain
        upload!(s)
        set_theta!(s, sys.param.θ)
        for _ in 1:sys.param.Tmax
            callback_iteration!(sys, s, f, measure)
        end
        download!(s)
    else
        upload!(s)
        twin = GB300State(s.sys; plain = true)
        fout = Array{Float64}(undef, s.sys.Lx, s.sys.Ly, 9)
        get_field!(fout, s, FIELD_FOUT)
        set_field!(twin, FIELD_FOUT, fout)
        twin.height .= s.height; twin.velx .= s.velx; twin.vely .= s.vely
        upload!(twin)
        set_theta!(twin, sys.param.θ)
        for _ in 1:sys.param.Tmax
            callback_iteration!(sys, twin, f, measure)
        end
        get_field!(fout, twin, FIELD_FOUT)
        set_field!(s, FIELD_FOUT, fout)
        download!(twin)
        s.height .= twin.height; s.velx .= twin.velx; s.vely .= twin.vely
        upload!(s)
    end
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
# inclination!(α, state; t, tstart, tsmooth) (src/forcing.jl:363-368): Fx .+= h α₁ (...)
Swalbe.inclination!(α::Vector, s::GB300State; t = 1000, tstart = 0, tsmooth = 1) =
    check(ccall((:swb_op_inclination, libswb), Cint,
                (Ptr{Cvoid}, Cdouble, Cdouble, Int64, Int64, Int64), s.handle, α[1], α[2], t,
                tstart, tsmooth), s.handle)

# ------------------------------------------------------------------ ensembles
"""
    GB300Batch(systems; T = Float32)

Many lattices of uneven size and parameters, advanced together by one launch
per time step over all of them (swb_batch_*): the GPU form of a loop of
independent simulations.  Lattice `i` (1-based) starts from height 1 until
`set_height!` gives it a film.
"""
mutable struct GB300Batch
    handle::Ptr{Cvoid}
    systems::Vector{Swalbe.SysConst}
end

function GB300Batch(systems::AbstractVector{<:Swalbe.SysConst}; T = Float32)
    params = [SwbParams(s) for s in systems]
    ref = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:swb_batch_create, libswb), Cint, (Ptr{SwbParams}, Cint, Cint, Ref{Ptr{Cvoid}}),
                params, length(params), PRECISION[T], ref), C_NULL)
    b = GB300Batch(ref[], collect(systems))
    finalizer(b) do x
        x.handle == C_NULL || ccall((:swb_batch_destroy, libswb), Cint, (Ptr{Cvoid},), x.handle)
        x.handle = C_NULL
    end
    return b
end

set_height!(b::GB300Batch, i::Integer, h::AbstractMatrix) =
    check(ccall((:swb_batch_set_height, libswb), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}),
                b.handle, i - 1, Matrix{Float64}(h)), C_NULL)

function height(b::GB300Batch, i::Integer)
    sys = b.systems[i]
    h = zeros(sys.Lx, sys.Ly)
    check(ccall((:swb_batch_get_height, libswb), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}),
                b.handle, i - 1, h), C_NULL)
    return h
end

# θ(x, t) = θ0 + Δθ sin(2π(x - v t)/Lx) for lattice i (moving wettability)
set_theta_wave!(b::GB300Batch, i::Integer, θ0, Δθ, v) =
    check(ccall((:swb_batch_set_theta_wave, libswb), Cint,
                (Ptr{Cvoid}, Cint, Cdouble, Cdouble, Cdouble), b.handle, i - 1, θ0, Δθ, v), C_NULL)

# strips of every lattice (default: chosen by timing real steps)
set_geometry!(b::GB300Batch, nt::Integer, rows::Integer) =
    check(ccall((:swb_batch_set_geometry, libswb), Cint, (Ptr{Cvoid}, Cint, Cint), b.handle, nt,
                rows), C_NULL)

function step!(b::GB300Batch, n::Integer)
    check(ccall((:swb_batch_step, libswb), Cint, (Ptr{Cvoid}, Int64), b.handle, n), C_NULL)
    check(ccall((:swb_batch_sync, libswb), Cint, (Ptr{Cvoid},), b.handle), C_NULL)
end

# ------------------------------------------------------------------ serving
# swb_request_info: the same field order and C types (Int32 then padding)
struct SwbRequestInfo
    id::Int64
    status::Int32
    steps_done::Int64
    t_submit::Float64
    t_admit::Float64
    t_done::Float64
end

"""
    GB300Server(hbm_budget; T = Float32, steps_per_tick = 100)

A request loop (swb_server_*): solves are admitted while their device memory
fits `hbm_budget` bytes and advanced together, `steps_per_tick` time steps
per scheduling tick; `submit` queues one, `poll` returns its height when it
is done.
"""
mutable struct GB300Server
    handle::Ptr{Cvoid}
end

function GB300Server(hbm_budget::Integer; T = Float32, steps_per_tick::Integer = 100)
    ref = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:swb_server_create, libswb), Cint, (Csize_t, Cint, Cint, Ref{Ptr{Cvoid}}),
                hbm_budget, PRECISION[T], steps_per_tick, ref), C_NULL)
    sv = GB300Server(ref[])
    finalizer(sv) do x
        x.handle == C_NULL || ccall((:swb_server_destroy, libswb), Cint, (Ptr{Cvoid},), x.handle)
        x.handle = C_NULL
    end
    return sv
end

# :fifo or :sjf (shortest job first), and an optional bound on resident cells
set_policy!(sv::GB300Server, policy::Symbol; max_resident_cells::Integer = 0) =
    check(ccall((:swb_server_set_policy, libswb), Cint, (Ptr{Cvoid}, Cint, Int64), sv.handle,
                policy === :sjf ? 1 : 0, max_resident_cells), C_NULL)

set_queue_limit!(sv::GB300Server, n::Integer) =
    check(ccall((:swb_server_set_queue_limit, libswb), Cint, (Ptr{Cvoid}, Int64), sv.handle, n),
          C_NULL)

# strips of the resident set (nt = 0: chosen per set)
set_geometry!(sv::GB300Server, nt::Integer = 0, rows::Integer = 0) =
    check(ccall((:swb_server_set_geometry, libswb), Cint, (Ptr{Cvoid}, Cint, Cint), sv.handle, nt,
                rows), C_NULL)

"""
    submit(sv, sys, h0, nsteps; θ0 = sys.param.θ, Δθ = 0, v = 0)

Queues a solve of `nsteps` time steps from the film `h0` (moving wettability
when Δθ or v is not 0).  Returns its id, or `nothing` when the queue is full.
"""
function submit(sv::GB300Server, sys::Swalbe.SysConst, h0::AbstractMatrix, nsteps::Integer;
                θ0 = sys.param.θ, Δθ = 0.0, v = 0.0)
    id = Ref{Int64}(0)
    st = ccall((:swb_server_submit, libswb), Cint,
               (Ptr{Cvoid}, Ref{SwbParams}, Ptr{Float64}, Cdouble, Cdouble, Cdouble, Int64,
                Ref{Int64}), sv.handle, Ref(SwbParams(sys)), Matrix{Float64}(h0), θ0, Δθ, v,
               nsteps, id)
    st == SWB_ERR_BUSY && return nothing
    check(st, C_NULL)
    return id[]
end

"""
    poll(sv, id, sys) -> (done, height or nothing, info)

A failed or cancelled request is reported through `info.status < 0`.
"""
function poll(sv::GB300Server, id::Integer, sys::Swalbe.SysConst)
    h = zeros(sys.Lx, sys.Ly)
    info = Ref{SwbRequestInfo}()
    st = ccall((:swb_server_poll, libswb), Cint,
               (Ptr{Cvoid}, Int64, Ptr{Float64}, Ref{SwbRequestInfo}), sv.handle, id, h, info)
    (st == SWB_ERR_ARG || st == SWB_ERR_NOT_FOUND) && check(st, C_NULL)
    return st == 1, (st == 1 ? h : nothing), info[]
end

cancel!(sv::GB300Server, id::Integer) =
    check(ccall((:swb_server_cancel, libswb), Cint, (Ptr{Cvoid}, Int64), sv.handle, id), C_NULL)

end  # module
