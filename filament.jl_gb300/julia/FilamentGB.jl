# FilamentGB.jl -- ccall binding of libfilament_gb.so for Filament.jl.
# Mirrors include/filament_gb.h; `run!` replaces the step loop of
# Filament.main_loop (src/Filament.jl:111-184).  Not executed in this
# environment (no Julia); the Python binding filament_gb/_abi.py is the
# tested twin.
module FilamentGB
const LIB = joinpath(@__DIR__, "..", "_build", "libfilament_gb.so")

# mirrors fil_config / fil_tables / fil_stats of include/filament_gb.h field by field
struct FilConfig
    abi_version::Int32; geometry::Int32; precision::Int32; alg::Int32
    n1::Int32; n2::Int32; nt::Int32
    nonlinearity::Int32; plasma::Int32; kparaxial::Int32; qparaxial::Int32
    resp_mask::UInt32; cubic_thg::Int32; losses_ereal::Int32; raman_thg::Int32
    plasma_alg::Int32; plasma_ereal::Int32; plasma_kdep::Int32; plasma_ncomp::Int32
    rate_n::Int32; reserved_i::NTuple{8,Int32}
    dt::Float64; dz0::Float64; phimax::Float64; phik::Float64; phip::Float64
    istop::Float64; rho0::Float64; dxdy::Float64; reserved_d::NTuple{8,Float64}
end
struct FilTables            # 25 pointers, in header order; C_NULL for absent tables
    p::NTuple{25,Ptr{Float64}}
end
struct FilStats
    z::Float64; dz::Float64; imax::Float64; rhomax::Float64; energy::Float64
    steps::Int64; status::Int32; flags::Int32
end

function create(cfg::FilConfig, tab::FilTables)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    rc = ccall((:fil_create, LIB), Cint, (Ref{FilConfig}, Ref{FilTables}, Ref{Ptr{Cvoid}}), cfg, tab, h)
    rc < 0 && error(unsafe_string(ccall((:fil_last_error, LIB), Cstring, (Ptr{Cvoid},), C_NULL)))
    return h[]
end
destroy(h) = ccall((:fil_destroy, LIB), Cint, (Ptr{Cvoid},), h)
set_field(h, E::Array{ComplexF64}) =                     # column-major E[Nr, Nt], real signal
    ccall((:fil_set_field, LIB), Cint, (Ptr{Cvoid}, Ptr{ComplexF64}, Cint, Cint, Cint), h, E, 1, 0, 0)
zstep(h, z, dz) = ccall((:fil_step, LIB), Cint, (Ptr{Cvoid}, Cdouble, Cdouble), h, z, dz)
function run!(h, z0, zmax, nmax)
    st = Ref{FilStats}()
    rc = ccall((:fil_run, LIB), Cint, (Ptr{Cvoid}, Cdouble, Cdouble, Int64, Ref{FilStats}), h, z0, zmax, nmax, st)
    return rc, st[]
end
analyze(h, F, P, rho_end) = ccall((:fil_analyze, LIB), Cint,
    (Ptr{Cvoid}, Ptr{FilStats}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}), h, C_NULL, F, P, rho_end)
get_field!(h, E::Array{ComplexF64}) =
    ccall((:fil_get_field, LIB), Cint, (Ptr{Cvoid}, Ptr{ComplexF64}, Cint, Cint), h, E, 1, 0)
# FieldAnalyzers.jl:180-197 / 320-336: the integral power spectrum S (Nt/2 + 1 bins)
function spectrum(h, nt)
    S = zeros(nt ÷ 2 + 1)
    ccall((:fil_analyze_spectrum, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}, Cint), h, S, length(S))
    return S
end
# ALG = Tsit5() / ATsit5(): FIL_ALG_TSIT5 = 5, FIL_ALG_ATSIT5 = 6 in FilConfig.alg;
# ATsit5 tolerances (option 7 rtol, 8 atol, value = tol * 1e12) and substep counts
set_option(h, opt, value) = ccall((:fil_set_option, LIB), Cint, (Ptr{Cvoid}, Cint, Int64), h, opt, value)
function ode_stats(h)
    out = zeros(Int64, 2)
    ccall((:fil_get_ode_stats, LIB), Cint, (Ptr{Cvoid}, Ptr{Int64}), h, out)
    return out[1], out[2]
end
# learned plasma surrogate counters: armed, in use, steps, steps that used the
# network, checks, failed checks, last and largest check error, mean rows and
# mean 128-point tiles per step that used the network
const SURROGATE_STAT_KEYS = (:armed, :in_use, :steps, :steps_used, :checks, :checks_failed,
                             :err_last, :err_max, :rows_mean, :tiles_mean)
function surrogate_stats(h)
    out = zeros(length(SURROGATE_STAT_KEYS))
    ccall((:fil_get_surrogate_stats, LIB), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Cint), h, out, length(out))
    return NamedTuple{SURROGATE_STAT_KEYS}(Tuple(out))
end

# batched sweep: members on uneven grids, one CUDA graph per z-step
function create_batch(cfgs::Vector{FilConfig}, tabs::Vector{FilTables})
    b = Ref{Ptr{Cvoid}}(C_NULL)
    rc = ccall((:fil_create_batch, LIB), Cint, (Cint, Ptr{FilConfig}, Ptr{FilTables}, Ref{Ptr{Cvoid}}),
               length(cfgs), cfgs, tabs, b)
    rc < 0 && error(unsafe_string(ccall((:fil_batch_last_error, LIB), Cstring, (Ptr{Cvoid},), C_NULL)))
    return b[]
end
batch_member(b, i) = ccall((:fil_batch_member, LIB), Ptr{Cvoid}, (Ptr{Cvoid}, Cint), b, i - 1)
function batch_tune!(b, max_branches=16)
    ms = zeros(8)
    ccall((:fil_batch_tune, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Cint), b, max_branches, ms, 8)
    return ms
end
function batch_run!(b, z0::Vector{Float64}, zmax::Vector{Float64}, nmax)
    st = Vector{FilStats}(undef, length(z0))
    rc = ccall((:fil_batch_run, LIB), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Int64, Ptr{FilStats}),
               b, z0, zmax, nmax, st)
    return rc, st
end
batch_destroy(b) = ccall((:fil_batch_destroy, LIB), Cint, (Ptr{Cvoid},), b)
end
