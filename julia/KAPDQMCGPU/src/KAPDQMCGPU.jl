"""
    KAPDQMCGPU

Julia binding of libkapdqmc_gpu.so: `phy_update` methods for KAPDQMC's
`tU_Hubbard_Para_`, `tV_Hubbard_Para_` and `tUV_Hubbard_Para_` that run the
sweep on a GB300 through the C ABI in include/kapdqmc.h.  The model structs
and their keyword constructors are KAPDQMC's own (src/tU/model.jl,
src/tV/model.jl, src/tUV/model.jl); only the sweep moves to the GPU.

    using KAPDQMC, KAPDQMCGPU
    model = tU_Hubbard_Para(Ht=1.0, Hu1=4.0, Hu2=4.0, Δt=0.1, Θrelax=5.0, Θquench=0.0,
                            Lattice="SQUARE45", site=[2, 4], BatchSize=10, Initial="H0")
    s = Initial_s(model, MersenneTwister(1234))
    s = KAPDQMCGPU.phy_update(path, model, s, 10, true)          # one chain
    ss = KAPDQMCGPU.phy_update(path, model, [s1, s2, ...], 10, true)  # a batch of chains

Keyword options (none changes the positional signature of the reference,
src/tU/phy_update.jl:3): `seed` (Philox stream; default time-based like the
reference's generator), `tape = (k, u)` (explicit proposal tape: per
proposal a choice index 0..2 and a uniform in [0,1), in the reference's
consumption order), `device`.
"""
module KAPDQMCGPU

using KAPDQMC
using DelimitedFiles
using Random

const libkdq = get(ENV, "KAPDQMC_GPU_LIB",
                   joinpath(@__DIR__, "..", "..", "..", "kapdqmc_gb300", "libkapdqmc_gpu.so"))

const KDQ_TU, KDQ_TV, KDQ_TUV = Int32(0), Int32(1), Int32(2)
const LATTICE_ID = Dict("SQUARE45" => Int32(0), "SQUARE90" => Int32(1),
                        "HoneyComb120" => Int32(2), "HoneyComb60" => Int32(3))

# kdq_model_desc, field for field
struct KdqModelDesc
    kind::Int32
    lattice::Int32
    site1::Int32
    site2::Int32
    Ns::Int32
    Nt::Int32
    z::Int32
    g_complex::Int32
    k_complex::Int32
    n_nodes::Int32
    nodes::Ptr{Int64}
    alpha::Ptr{Float64}
    gamma::Ptr{Float64}
    eta::Ptr{Float64}
    a::Float64
    Ht::Float64
    U::Float64
    V::Float64
    eK::Ptr{Float64}
    eKinv::Ptr{Float64}
    HalfeK::Ptr{Float64}
    HalfeKinv::Ptr{Float64}
    K::Ptr{Float64}
    Pt::Ptr{Float64}
    bonds::Ptr{Int32}
end

check(rc, h) = rc == 0 || error("kapdqmc: ", unsafe_string(ccall((:kdq_last_error, libkdq), Cstring, (Ptr{Cvoid},), h)))

# complex matrices travel as interleaved Float64, real ones as Float64
flat(A, cplx::Bool) = cplx ? collect(reinterpret(Float64, vec(ComplexF64.(A)))) : Float64.(real.(vec(A)))

function bond_list(nnidx)
    b = Vector{Int32}(undef, 2 * length(nnidx))
    for (q, (x, y)) in enumerate(nnidx)        # column-major order of nnidx
        b[2q-1] = x
        b[2q] = y
    end
    b
end

kind_of(::KAPDQMC.tUDQMC.tU_Hubbard_Para_) = KDQ_TU
kind_of(::KAPDQMC.tVDQMC.tV_Hubbard_Para_) = KDQ_TV
kind_of(::KAPDQMC.tUVDQMC.tUV_Hubbard_Para_) = KDQ_TUV

g_complex(m::KAPDQMC.tUVDQMC.tUV_Hubbard_Para_) = m.Type == ComplexF64
g_complex(m::KAPDQMC.tUDQMC.tU_Hubbard_Para_) = true
g_complex(m::KAPDQMC.tVDQMC.tV_Hubbard_Para_) = false

"""Create a handle with `nchains` chains; returns (handle, n_obs)."""
function create(model, nchains::Integer; device::Integer=0)
    kind = kind_of(model)
    gc = g_complex(model)
    kc = any(M -> eltype(M) <: Complex && any(!iszero, imag.(M)),
             (model.eK, model.eKinv, model.HalfeK, model.HalfeKinv, model.K))
    nodes = Int64.(model.nodes)
    alpha = kind == KDQ_TUV ? Float64[] : Float64.(model.α)
    gamma, eta = Float64.(model.γ), Float64.(model.η)
    mats = [flat(M, kc) for M in (model.eK, model.eKinv, model.HalfeK, model.HalfeKinv, model.K)]
    pt = flat(model.Pt, gc)
    bonds = kind == KDQ_TU ? Int32[] : bond_list(model.nnidx)
    z = kind == KDQ_TU ? 1 : size(model.nnidx, 2)
    site2 = length(model.site) > 1 ? model.site[2] : 1
    a = kind == KDQ_TUV ? model.a : 0.0
    U = kind == KDQ_TUV ? model.U : 0.0
    V = kind == KDQ_TUV ? model.V : 0.0
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve nodes alpha gamma eta mats pt bonds begin
        d = KdqModelDesc(kind, LATTICE_ID[model.Lattice], model.site[1], site2, model.Ns, model.Nt, z,
                         gc, kc, length(nodes), pointer(nodes),
                         isempty(alpha) ? Ptr{Float64}(C_NULL) : pointer(alpha),
                         pointer(gamma), pointer(eta), a, model.Ht, U, V,
                         pointer(mats[1]), pointer(mats[2]), pointer(mats[3]), pointer(mats[4]),
                         pointer(mats[5]), pointer(pt),
                         isempty(bonds) ? Ptr{Int32}(C_NULL) : pointer(bonds))
        rc = ccall((:kdq_create, libkdq), Cint, (Ref{Ptr{Cvoid}}, Ref{KdqModelDesc}, Int32, Int32),
                   h, d, nchains, device)
        rc == 0 || error("kapdqmc: ", unsafe_string(ccall((:kdq_last_error, libkdq), Cstring, (Ptr{Cvoid},), C_NULL)))
    end
    n_obs = ccall((:kdq_n_obs, libkdq), Cint, (Ptr{Cvoid},), h[])
    return h[], n_obs
end

destroy(h) = ccall((:kdq_destroy, libkdq), Cvoid, (Ptr{Cvoid},), h)

"""
    phy_update(path, model, s, Sweeps, record=false; seed, tape, device)

GPU replacement of the reference's `phy_update` (src/tU/phy_update.jl:3-152,
src/tV/phy_update.jl:1-188, src/tUV/phy_update.jl:1-186).  `s` is one field
(returned updated, as in the reference) or a vector of fields (one chain
each).  With `record`, one CSV row per sweep, averaged over the chains, is
appended to the reference's file name under `path`.
"""
function phy_update(path::String, model, s, Sweeps::Int64, record::Bool=false;
                    seed::Union{Nothing,Integer}=nothing, tape=nothing, device::Integer=0,
                    autotune::Bool=false)
    fields = s isa AbstractVector{<:AbstractArray} ? s : [s]
    nch = length(fields)
    h, n_obs = create(model, nch; device=device)
    try
        buf = reduce(vcat, [vec(UInt8.(f)) for f in fields])
        check(ccall((:kdq_set_fields, libkdq), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), h, buf, length(buf)), h)
        if tape === nothing
            sd = seed === nothing ? time_ns() : UInt64(seed)
            check(ccall((:kdq_set_rng, libkdq), Cint, (Ptr{Cvoid}, UInt64, UInt64), h, sd, 0), h)
        else
            k, u = tape
            check(ccall((:kdq_set_tape, libkdq), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Ptr{Float64}, Csize_t),
                        h, UInt8.(k), Float64.(u), length(k) ÷ nch), h)
        end
        if autotune   # pick the sweep kernel's tile class (state restored)
            check(ccall((:kdq_autotune, libkdq), Cint, (Ptr{Cvoid}, Ptr{Int32}, Ptr{Float64}, Int32),
                        h, C_NULL, C_NULL, 0), h)
        end
        obs = zeros(Float64, n_obs * Sweeps * nch)
        check(ccall((:kdq_phy_update, libkdq), Cint, (Ptr{Cvoid}, Int32, Int32, Ptr{Float64}, Csize_t),
                    h, Sweeps, record, obs, length(obs)), h)
        check(ccall((:kdq_get_fields, libkdq), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), h, buf, length(buf)), h)
        n = length(fields[1])
        for (c, f) in enumerate(fields)
            copyto!(f, reshape(buf[(c-1)*n+1:c*n], size(f)))
        end
        if record
            rows = reshape(obs, n_obs, Sweeps, nch)            # chain-major rows
            mean_rows = dropdims(sum(rows, dims=3), dims=3) ./ nch
            open(csv_name(path, model), "a") do io
                writedlm(io, permutedims(mean_rows), ',')
            end
        end
    finally
        destroy(h)
    end
    return s
end

"""
    reference_tape(model, s, rng::AbstractRNG, Sweeps) -> (k, u)

The proposal tape that the reference's own `phy_update` draws from `rng`
over `Sweeps` sweeps of one chain with field `s`, for `phy_update(...;
tape=(k, u))`: with `rng = MersenneTwister(seed)` patched into the
reference's driver in place of its clock-seeded generator
(src/tU/phy_update.jl:31, src/tV/phy_update.jl:25, src/tUV/phy_update.jl:24),
both runs consume the same random stream and must make the same accept /
reject decisions.  Each proposal of the reference takes exactly one
`rand(rng, model.samplers_dict[s_i])` and then one `rand(rng)`, accepted or
not (src/tU/phy_update.jl:259,262, src/tV/phy_update.jl:194,200,
src/tUV/phy_update.jl:192,198), and a sweep makes 2 proposals per field
entry (forward and backward over every slice).  Every sampler of
`samplers_dict` (src/tU/model.jl:87-93) draws an index into the ascending
3-element list of the values other than its key with the same call, so
drawing through the sampler of key 1 consumes the stream exactly as the
reference does whatever the current field; the drawn value v in {2, 3, 4}
is index v - 2 of that list, which is the tape's choice index k (the k-th
of {1,2,3,4} without the current value, ascending).  For a batch of chains,
concatenate the chains' tapes chain by chain.  Not yet run: no Julia
installation was available where this binding was written, so this helper
is untested.
"""
function reference_tape(model, s, rng::AbstractRNG, Sweeps::Integer)
    n = 2 * length(s) * Sweeps
    k = Vector{UInt8}(undef, n)
    u = Vector{Float64}(undef, n)
    sp = model.samplers_dict[UInt8(1)]
    for m in 1:n
        k[m] = UInt8(rand(rng, sp) - 2)
        u[m] = rand(rng)
    end
    return k, u
end

"""
    phy_update_group(path, models, ss, Sweeps, record=false; seed, device)

`phy_update` for several models at once (different lattices, models or
precisions): `models[i]` with the vector of fields `ss[i]` (one chain per
field, updated in place).  All chains are swept together, one CUDA graph per
sweep (`kdq_group_sweep`); every model's chains give the same results as a
`phy_update` of that model alone with the same seed.  With `record`, each
model's CSV file gets its rows as in `phy_update`.  No counterpart in the
reference, which runs one model per call.
"""
function phy_update_group(path::String, models::Vector, ss::Vector, Sweeps::Int64, record::Bool=false;
                          seed::Union{Nothing,Integer}=nothing, device::Integer=0)
    length(models) == length(ss) || error("one vector of fields per model")
    sd = seed === nothing ? time_ns() : UInt64(seed)
    hs = Ptr{Cvoid}[]
    nobs = Int[]
    g = Ref{Ptr{Cvoid}}(C_NULL)
    try
        for (i, (model, fields)) in enumerate(zip(models, ss))
            h, n_obs = create(model, length(fields); device=device)
            push!(hs, h)
            push!(nobs, n_obs)
            buf = reduce(vcat, [vec(UInt8.(f)) for f in fields])
            check(ccall((:kdq_set_fields, libkdq), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), h, buf, length(buf)), h)
            check(ccall((:kdq_set_rng, libkdq), Cint, (Ptr{Cvoid}, UInt64, UInt64), h, sd + (i - 1), 0), h)
            check(ccall((:kdq_init, libkdq), Cint, (Ptr{Cvoid},), h), h)
        end
        rc = ccall((:kdq_group_create, libkdq), Cint, (Ref{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}, Int32), g, hs, length(hs))
        rc == 0 || error("kapdqmc: ", unsafe_string(ccall((:kdq_last_error, libkdq), Cstring, (Ptr{Cvoid},), C_NULL)))
        gerr(rc) = rc == 0 || error("kapdqmc: ", unsafe_string(ccall((:kdq_group_last_error, libkdq), Cstring,
                                                                     (Ptr{Cvoid},), g[])))
        gerr(ccall((:kdq_group_sweep, libkdq), Cint, (Ptr{Cvoid}, Int32, Int32), g[], Sweeps, record))
        gerr(ccall((:kdq_group_synchronize, libkdq), Cint, (Ptr{Cvoid},), g[]))
        for (i, (model, fields)) in enumerate(zip(models, ss))
            h, nch = hs[i], length(fields)
            n = length(fields[1])
            buf = zeros(UInt8, n * nch)
            check(ccall((:kdq_get_fields, libkdq), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), h, buf, length(buf)), h)
            for (c, f) in enumerate(fields)
                copyto!(f, reshape(buf[(c-1)*n+1:c*n], size(f)))
            end
            if record
                obs = zeros(Float64, nobs[i] * Sweeps * nch)
                check(ccall((:kdq_get_obs, libkdq), Cint, (Ptr{Cvoid}, Ptr{Float64}, Csize_t), h, obs, length(obs)), h)
                rows = reshape(obs, nobs[i], Sweeps, nch)
                mean_rows = dropdims(sum(rows, dims=3), dims=3) ./ nch
                open(csv_name(path, model), "a") do io
                    writedlm(io, permutedims(mean_rows), ',')
                end
            end
        end
    finally
        g[] == C_NULL || ccall((:kdq_group_destroy, libkdq), Cvoid, (Ptr{Cvoid},), g[])
        foreach(destroy, hs)
    end
    return ss
end

"""
    ctrl_SCEEicr(path, model, indexA, indexB, Sweeps, λ, Nλ, ss, record; seed, device)

GPU replacement of the reference's coupled incremental SCEE sweep
(src/tU/SCEE.jl:1-211, src/tV/SCEE.jl:1-431, src/tUV/SCEE.jl:1-339).  `ss` is
the replica pair [s1, s2] (updated in place and returned); with `record` the
row λ, O_1, ..., O_Sweeps is appended to the reference's file name under `path`.
"""
function ctrl_SCEEicr(path::String, model, indexA::Vector{Int64}, indexB::Vector{Int64}, Sweeps::Int64,
                      λ::Float64, Nλ::Int64, ss, record; seed::Union{Nothing,Integer}=nothing, device::Integer=0)
    h, _ = create(model, 2; device=device)
    try
        buf = vcat(vec(UInt8.(ss[1])), vec(UInt8.(ss[2])))
        check(ccall((:kdq_set_fields, libkdq), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), h, buf, length(buf)), h)
        sd = seed === nothing ? time_ns() : UInt64(seed)
        check(ccall((:kdq_set_rng, libkdq), Cint, (Ptr{Cvoid}, UInt64, UInt64), h, sd, 0), h)
        check(ccall((:kdq_scee_enable, libkdq), Cint, (Ptr{Cvoid}, Ptr{Int32}, Int32, Ptr{Int32}, Int32, Float64, Int32),
                    h, Int32.(indexA), length(indexA), Int32.(indexB), length(indexB), λ, Nλ), h)
        O = zeros(Float64, Sweeps + 1)
        check(ccall((:kdq_scee_run, libkdq), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}, Csize_t), h, Sweeps, O, length(O)), h)
        check(ccall((:kdq_get_fields, libkdq), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), h, buf, length(buf)), h)
        n = length(ss[1])
        copyto!(ss[1], reshape(buf[1:n], size(ss[1])))
        copyto!(ss[2], reshape(buf[n+1:2n], size(ss[2])))
        if record
            open(scee_name(path, model, Nλ), "a") do io
                writedlm(io, O', ',')
            end
        end
    finally
        destroy(h)
    end
    return ss
end

"""
    ctrl_SCDOPicr(path, model, alpha, indexA, indexB, Sweeps, λ, Nλ, s, record; seed, device)

GPU replacement of the reference's disorder-operator sweep
(src/tU/disorder_operate.jl:1-247), t-U.
"""
function ctrl_SCDOPicr(path::String, model, alpha::Float64, indexA::Vector{Int64}, indexB::Vector{Int64},
                       Sweeps::Int64, λ::Float64, Nλ::Int64, s, record; seed::Union{Nothing,Integer}=nothing,
                       device::Integer=0)
    h, _ = create(model, 1; device=device)
    try
        buf = vec(UInt8.(s))
        check(ccall((:kdq_set_fields, libkdq), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), h, buf, length(buf)), h)
        sd = seed === nothing ? time_ns() : UInt64(seed)
        check(ccall((:kdq_set_rng, libkdq), Cint, (Ptr{Cvoid}, UInt64, UInt64), h, sd, 0), h)
        check(ccall((:kdq_dop_enable, libkdq), Cint,
                    (Ptr{Cvoid}, Float64, Ptr{Int32}, Int32, Ptr{Int32}, Int32, Float64, Int32),
                    h, alpha, Int32.(indexA), length(indexA), Int32.(indexB), length(indexB), λ, Nλ), h)
        O = zeros(Float64, Sweeps + 1)
        check(ccall((:kdq_dop_run, libkdq), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}, Csize_t), h, Sweeps, O, length(O)), h)
        check(ccall((:kdq_get_fields, libkdq), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), h, buf, length(buf)), h)
        copyto!(s, reshape(buf, size(s)))
        if record
            name = Dict("SQUARE90" => "□90", "SQUARE45" => "□45", "HoneyComb60" => "HC", "HoneyComb120" => "HC120")[model.Lattice]
            file = length(unique(model.α)) == 1 ?
                "$(path)/tUSCDOP$(name)_t$(model.Ht)U$(model.Hu1)size$(model.site)Δt$(model.Δt)Θ$(model.Θrelax)N$(Nλ)BS$(model.BatchSize).csv" :
                "$(path)/tUSCDOP$(name)_t$(model.Ht)U$(model.Hu1)_$(model.Hu2)size$(model.site)Δt$(model.Δt)Θ$(model.Θrelax)_$(model.Θquench)N$(Nλ)BS$(model.BatchSize).csv"
            open(file, "a") do io
                writedlm(io, O', ',')
            end
        end
    finally
        destroy(h)
    end
    return s
end

# SCEE CSV names (src/tU/SCEE.jl:16-32, src/tV/SCEE.jl:16-32, src/tUV/SCEE.jl:16-26)
function scee_name(path, model::KAPDQMC.tUDQMC.tU_Hubbard_Para_, Nλ)
    name = Dict("SQUARE90" => "□90", "SQUARE45" => "□45", "HoneyComb60" => "HC", "HoneyComb120" => "HC120")[model.Lattice]
    model.Θquench == 0.0 ?
        "$(path)/tUSCEE$(name)_t$(model.Ht)U$(model.Hu1)size$(model.site)Δt$(model.Δt)Θ$(model.Θrelax)N$(Nλ)BS$(model.BatchSize).csv" :
        "$(path)/tUSCEE$(name)_t$(model.Ht)U$(model.Hu1)_$(model.Hu2)size$(model.site)Δt$(model.Δt)Θ$(model.Θrelax)_$(model.Θquench)N$(Nλ)BS$(model.BatchSize).csv"
end
function scee_name(path, model::KAPDQMC.tVDQMC.tV_Hubbard_Para_, Nλ)
    name = occursin("SQUARE", model.Lattice) ? "□" : (model.Lattice == "HoneyComb60" ? "HC" : "HC120")
    length(unique(model.α)) == 1 ?
        "$(path)/tVSCEE$(name)_t$(model.Ht)V$(model.Hv1)size$(model.site)Δt$(model.Δt)Θ$(model.Θrelax)N$(Nλ)BS$(model.BatchSize).csv" :
        "$(path)/tVSCEE$(name)_t$(model.Ht)V$(model.Hv1)_$(model.Hv2)size$(model.site)Δt$(model.Δt)Θ$(model.Θrelax)_$(model.Θquench)N$(Nλ)BS$(model.BatchSize).csv"
end
function scee_name(path, model::KAPDQMC.tUVDQMC.tUV_Hubbard_Para_, Nλ)
    name = occursin("SQUARE", model.Lattice) ? "□" : (model.Lattice == "HoneyComb60" ? "HC60" : "HC120")
    "$(path)/tUVSCEE$(name)_t$(model.Ht)U$(model.U)V$(model.V)size$(model.site)Δt$(model.Δt)Θ$(model.Θ)N$(Nλ)BS$(model.BatchSize).csv"
end

# CSV names of the reference (src/tU/phy_update.jl:12-27, src/tV/phy_update.jl:10-23,
# src/tUV/phy_update.jl:13-22)
function csv_name(path, model::KAPDQMC.tUDQMC.tU_Hubbard_Para_)
    name = Dict("SQUARE90" => "□90", "SQUARE45" => "□45", "HoneyComb60" => "HC", "HoneyComb120" => "HC120")[model.Lattice]
    model.Θquench == 0.0 ?
        "$(path)/tUphy$(name)_t$(model.Ht)U$(model.Hu1)size$(model.site)Δt$(model.Δt)Θ$(model.Θrelax)BS$(model.BatchSize).csv" :
        "$(path)/tUphy$(name)_t$(model.Ht)U$(model.Hu1)_$(model.Hu2)size$(model.site)Δt$(model.Δt)Θ$(model.Θrelax)_$(model.Θquench)BS$(model.BatchSize).csv"
end
function csv_name(path, model::KAPDQMC.tVDQMC.tV_Hubbard_Para_)
    name = occursin("SQUARE", model.Lattice) ? "□" : (model.Lattice == "HoneyComb60" ? "HC" : "HC120")
    length(unique(model.α)) == 1 ?
        "$(path)/tVphy$(name)_t$(model.Ht)V$(model.Hv1)size$(model.site)Δt$(model.Δt)Θ$(model.Θrelax)BS$(model.BatchSize).csv" :
        "$(path)/tVphy$(name)_t$(model.Ht)V$(model.Hv1)_$(model.Hv2)size$(model.site)Δt$(model.Δt)Θ$(model.Θrelax)_$(model.Θquench)BS$(model.BatchSize).csv"
end
function csv_name(path, model::KAPDQMC.tUVDQMC.tUV_Hubbard_Para_)
    name = occursin("SQUARE", model.Lattice) ? "□" : (model.Lattice == "HoneyComb60" ? "HC" : "HC120")
    "$(path)/tUVphy$(name)_t$(model.Ht)U$(model.U)V$(model.V)size$(model.site)Δt$(model.Δt)Θ$(model.Θ)BS$(model.BatchSize).csv"
end

end # module
