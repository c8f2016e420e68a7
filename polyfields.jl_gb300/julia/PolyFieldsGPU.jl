# PolyFieldsGPU — runs PolyFields.jl's `scft!(sys, AndersonUpdater; domain, opts)` on a GB300
# through libpolyfields_gpu.so (C ABI: include/polyfields_gpu.h).
#
#     using PolyFields, PolyFieldsGPU
#     scft!(sys, AndersonUpdater(; nhist = 10); domain = DomainUpdater(; nskip = 5, nper = 20), opts = opts)
#
# The method below is more specific than PolyFields.scft!(::FieldSystem, ::AbstractFieldUpdater;
# ...) (src/simulate.jl:60-61), so user scripts run unchanged.  `precision = 1,
# mixed_switch_ferr = 1e-5` selects float32 propagators with a float64 polish.
#
# Status: written against the header and the reference's types (FieldSystem, Multiblock,
# Point, FloryInteraction, AndersonUpdater, DomainUpdater, SCFTOptions, SCFTResults); Julia is
# not installed where this library was built and tested, so this module has not been run.  The
# same entry points, with the same arguments, are exercised by the Python mirror in
# polyfields.jl_gb300/polyfields/ and its tests.
module PolyFieldsGPU

using PolyFields
import PolyFields: scft!
using ChainRulesCore

export scft_batch!, propagate_noalloc!

const lib = get(ENV, "POLYFIELDS_GPU_LIB", joinpath(@__DIR__, "..", "polyfields", "libpolyfields_gpu.so"))

struct PFOptions            # pf_scft_options
    nsteps::Cint
    nsout::Cint
    nsave::Cint
    polish::Cint              # 0 automatic, 1 float64 field-updater steps, 2 Newton-Krylov polish
    ftol::Cdouble
    stol::Cdouble
    mixed_switch_ferr::Cdouble
end

mutable struct PFResults    # pf_scft_results
    time::Cdouble
    nsteps::Cint
    converged::Cint
    ferr::Cdouble
    serr::Cdouble
    fhelm::Cdouble
    switch_step::Cint
    polish_fp64_solves::Cint
    polish_fp32_solves::Cint
    pad0::Cint
    PFResults() = new(0, 0, 0, 0, 0, 0, -1, 0, 0, 0)
end

const PF_OK, PF_EARG, PF_ECUDA, PF_ENAN, PF_ESINGULAR, PF_ETIMEOUT = 0, 1, 2, 3, 4, 5
const PF_FIELD, PF_DENSITY, PF_RESIDUAL, PF_POTENTIAL, PF_FIELD_COTANGENT = 0, 1, 2, 3, 4

# The engine's messages are the reference's error strings ("Diverging field updater --
# breaking.", "Error inverting Umn matrix ...", validation messages).
function check(h, st)
    st == PF_OK && return nothing
    msg = h == C_NULL ? unsafe_string(ccall((:pf_status_string, lib), Cstring, (Cint,), st)) :
          unsafe_string(ccall((:pf_last_error, lib), Cstring, (Ptr{Cvoid},), h))
    st == PF_EARG ? throw(ArgumentError(msg)) : error(msg)
end

# Device-side FieldSystem built from the Julia one; the fields are copied, Julia keeps ownership.
function gpu_system(sys::FieldSystem; precision::Integer = 0)
    ref = Ref{Ptr{Cvoid}}(C_NULL)
    nx, ny, nz = sys.dims
    check(C_NULL, ccall((:pf_system_create, lib), Cint, (Ref{Ptr{Cvoid}}, Cint, Cint, Cint, Cint),
                        ref, nx, ny, nz, precision))
    h = ref[]
    c = sys.cell
    check(h, ccall((:pf_set_cell, lib), Cint, (Ptr{Cvoid}, Cint, Cstring, Ptr{Cdouble}, Cint),
                   h, c.dim, String(c.crystal), collect(Float64, c.params), length(c.params)))
    for mid in sort(collect(keys(sys.monomers)))
        m = sys.monomers[mid]
        check(h, ccall((:pf_add_monomer, lib), Cint, (Ptr{Cvoid}, Cint, Cdouble, Cdouble), h, m.id, m.vol, m.charge))
    end
    for (isp, sp) in enumerate(sys.species)
        phi = sys.phi_species[isp]
        if sp isa Multiblock
            check(h, ccall((:pf_add_multiblock, lib), Cint,
                           (Ptr{Cvoid}, Cint, Ptr{Cint}, Ptr{Cint}, Ptr{Cdouble}, Cint, Cdouble),
                           h, length(sp.N_block), Cint.(sp.mid_block), Cint.(sp.N_block),
                           collect(Float64, sp.b_block), sp.Ns, phi))
        elseif sp isa Point
            check(h, ccall((:pf_add_point, lib), Cint, (Ptr{Cvoid}, Cint, Cdouble), h, sp.mids[1], phi))
        end
    end
    for itx in sys.interactions
        if itx isa FloryInteraction
            for ((a, b), chi) in itx.chis
                check(h, ccall((:pf_set_flory, lib), Cint, (Ptr{Cvoid}, Cint, Cint, Cdouble), h, a, b, chi))
            end
        elseif itx isa EdwardsInteraction
            for (mid, u) in itx.uvals
                check(h, ccall((:pf_set_edwards, lib), Cint, (Ptr{Cvoid}, Cint, Cdouble), h, mid, u))
            end
        end
    end
    for (mid, w) in sys.fields          # Array{Float64,3}[x, y, z] is x fastest: passed as is
        GC.@preserve w check(h, ccall((:pf_set_field, lib), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}), h, mid, w))
    end
    return h
end

function add_updaters!(h, u::AndersonUpdater, domain)
    check(h, ccall((:pf_anderson_create, lib), Cint, (Ptr{Cvoid}, Cint, Cint, Cdouble),
                   h, u.nhist, u.iter_euler, u.lam_euler))
    if domain !== nothing
        check(h, ccall((:pf_domain_create, lib), Cint, (Ptr{Cvoid}, Cint, Cint, Cdouble, Cdouble, Cdouble),
                       h, domain.nper, domain.nskip, domain.lam, domain.pmax, domain.rlxn))
    end
end

# Copy the engine's state back into the Julia FieldSystem (fields, densities, residuals,
# potentials and the cell parameters).
function pull_state!(sys::FieldSystem, h)
    for mid in keys(sys.fields)
        for (kind, dict) in ((PF_FIELD, sys.fields), (PF_DENSITY, sys.density), (PF_RESIDUAL, sys.residuals),
                             (PF_POTENTIAL, sys.potentials))
            a = dict[mid]
            GC.@preserve a check(h, ccall((:pf_get_grid, lib), Cint, (Ptr{Cvoid}, Cint, Cint, Ptr{Cdouble}),
                                          h, kind, mid, a))
        end
    end
    p = collect(Float64, sys.cell.params)
    check(h, ccall((:pf_get_cell, lib), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Cint, Ptr{Cdouble}),
                   h, p, length(p), Ref(0.0)))
    sys.cell.params .= p
    PolyFields.update!(sys.cell)
    return sys
end

pf_options(opts::SCFTOptions, mixed_switch_ferr; polish::Integer = 0) =
    PFOptions(opts.nsteps, opts.nsout, opts.nsave, polish, opts.ftol, opts.stol, mixed_switch_ferr)

# scft!(sys, AndersonUpdater; domain, opts) on the GPU (src/simulate.jl:60-148).
function scft!(sys::FieldSystem, u::AndersonUpdater; domain = nothing, opts::SCFTOptions = SCFTOptions(),
               precision::Integer = 0, mixed_switch_ferr::Real = 0.0)
    h = gpu_system(sys; precision)
    try
        add_updaters!(h, u, domain)
        o = pf_options(opts, mixed_switch_ferr)
        r = PFResults()
        # nsave checkpoints (simulate.jl:124-128): the engine writes savefields' JSON itself
        check(h, ccall((:pf_set_savepath, lib), Cint, (Ptr{Cvoid}, Cstring), h, opts.savepath))
        check(h, ccall((:pf_scft, lib), Cint, (Ptr{Cvoid}, Ref{PFOptions}, Cint, Ref{PFResults}),
                       h, o, domain === nothing ? 0 : 1, r))
        pull_state!(sys, h)
        return SCFTResults(r.time, r.nsteps, r.converged != 0, r.ferr, r.serr, r.fhelm)
    finally
        ccall((:pf_system_destroy, lib), Cint, (Ptr{Cvoid},), h)
    end
end

# Many independent scft! runs at once (a phase-diagram sweep): one handle per system, each on
# its own CUDA stream, nthreads host threads (pf_scft_batch).  Returns the SCFTResults and the
# per-system status (0 = ok; otherwise the error of that system only).
function scft_batch!(systems::Vector{<:FieldSystem}, u::AndersonUpdater; domain = nothing,
                     opts::SCFTOptions = SCFTOptions(), precision::Integer = 1, mixed_switch_ferr::Real = 1e-5,
                     nthreads::Integer = 32)
    hs = [gpu_system(s; precision) for s in systems]
    try
        for h in hs
            add_updaters!(h, u, domain)
        end
        o = pf_options(opts, mixed_switch_ferr)
        res = [PFResults() for _ in hs]
        st = zeros(Cint, length(hs))
        ccall((:pf_scft_batch, lib), Cint, (Ptr{Ptr{Cvoid}}, Cint, Ref{PFOptions}, Cint, Ptr{PFResults},
              Ptr{Cint}, Cint), hs, length(hs), o, domain === nothing ? 0 : 1, res, st, nthreads)
        out = SCFTResults[]
        for (i, (sys, h)) in enumerate(zip(systems, hs))
            st[i] == PF_OK && pull_state!(sys, h)
            r = res[i]
            push!(out, SCFTResults(r.time, r.nsteps, r.converged != 0, r.ferr, r.serr, r.fhelm))
        end
        return out, st
    finally
        for h in hs
            ccall((:pf_system_destroy, lib), Cint, (Ptr{Cvoid},), h)
        end
    end
end

# density(sys, w): the pooled monomer densities for fields w, as a differentiable function.
function density(sys::FieldSystem, w::Dict{Int,Array{Float64,3}}; precision::Integer = 0)
    h = gpu_system(sys; precision)
    try
        return density_on(h, w)
    finally
        ccall((:pf_system_destroy, lib), Cint, (Ptr{Cvoid},), h)
    end
end

function density_on(h, w)
    for (mid, wm) in w
        GC.@preserve wm check(h, ccall((:pf_set_field, lib), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}), h, mid, wm))
    end
    check(h, ccall((:pf_density, lib), Cint, (Ptr{Cvoid},), h))
    rho = Dict(mid => similar(wm) for (mid, wm) in w)
    for (mid, r) in rho
        GC.@preserve r check(h, ccall((:pf_get_grid, lib), Cint, (Ptr{Cvoid}, Cint, Cint, Ptr{Cdouble}),
                                      h, PF_DENSITY, mid, r))
    end
    return rho
end

# The pullback of density!(sys) (pf_set_density_cotangent + pf_density_pullback): dL/dw per
# monomer, dL/dtheta of the cell parameters, dL/dNref of every Multiblock block.
function ChainRulesCore.rrule(::typeof(density), sys::FieldSystem, w::Dict{Int,Array{Float64,3}};
                              precision::Integer = 0)
    h = gpu_system(sys; precision)
    rho = density_on(h, w)
    function density_pullback(rho_bar)
        rb = unthunk(rho_bar)
        for mid in keys(w)
            if haskey(rb, mid)
                r = rb[mid]
                GC.@preserve r check(h, ccall((:pf_set_density_cotangent, lib), Cint,
                                              (Ptr{Cvoid}, Cint, Ptr{Cdouble}), h, mid, r))
            else
                check(h, ccall((:pf_set_density_cotangent, lib), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}),
                               h, mid, C_NULL))
            end
        end
        cell_bar = zeros(length(sys.cell.params))
        nblk = sum((length(sp.N_block) for sp in sys.species if sp isa Multiblock); init = 0)
        nref_bar = zeros(max(nblk, 1))
        check(h, ccall((:pf_density_pullback, lib), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint),
                       h, cell_bar, length(cell_bar), nref_bar, nblk))
        w_bar = Dict(mid => similar(wm) for (mid, wm) in w)
        for (mid, g) in w_bar
            GC.@preserve g check(h, ccall((:pf_get_grid, lib), Cint, (Ptr{Cvoid}, Cint, Cint, Ptr{Cdouble}),
                                          h, PF_FIELD_COTANGENT, mid, g))
        end
        ccall((:pf_system_destroy, lib), Cint, (Ptr{Cvoid},), h)
        return NoTangent(), Tangent{typeof(sys)}(; cell = cell_bar), w_bar
    end
    return rho, density_pullback
end

# free_energy(sys, w) as a differentiable function (pf_free_energy_pullback): the pullback gives
# dF/dw per monomer and, as the system's tangent, dF/dtheta (cell), dF/dNref_b (blocks), dF/dchi
# (Flory pairs in ascending id order) and dF/du (Edwards monomers in ascending id order).
function ChainRulesCore.rrule(::typeof(PolyFields.free_energy), sys::FieldSystem, w::Dict{Int,Array{Float64,3}};
                              precision::Integer = 0)
    h = gpu_system(sys; precision)
    for (mid, wm) in w
        GC.@preserve wm check(h, ccall((:pf_set_field, lib), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}), h, mid, wm))
    end
    np = length(sys.cell.params)
    nblk = sum((length(sp.N_block) for sp in sys.species if sp isa Multiblock); init = 0)
    pairs = sort(unique([p for itx in sys.interactions if itx isa FloryInteraction for p in keys(itx.chis)]))
    umids = sort(unique([m for itx in sys.interactions if itx isa EdwardsInteraction for m in keys(itx.uvals)]))
    cell_bar, nref_bar = zeros(max(np, 1)), zeros(max(nblk, 1))
    chi_bar, u_bar, f = zeros(max(length(pairs), 1)), zeros(max(length(umids), 1)), Ref(0.0)
    check(h, ccall((:pf_free_energy_pullback, lib), Cint,
                   (Ptr{Cvoid}, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint, Ref{Cdouble}),
                   h, cell_bar, np, nref_bar, nblk, chi_bar, length(pairs), u_bar, length(umids), f))
    w_bar = Dict(mid => similar(wm) for (mid, wm) in w)
    for (mid, g) in w_bar
        GC.@preserve g check(h, ccall((:pf_get_grid, lib), Cint, (Ptr{Cvoid}, Cint, Cint, Ptr{Cdouble}),
                                      h, PF_FIELD_COTANGENT, mid, g))
    end
    ccall((:pf_system_destroy, lib), Cint, (Ptr{Cvoid},), h)
    function free_energy_pullback(fbar)
        s = unthunk(fbar)
        tangent = Tangent{typeof(sys)}(; cell = s .* cell_bar[1:np], Nref_block = s .* nref_bar[1:nblk],
                                       chi = Dict(p => s * chi_bar[i] for (i, p) in enumerate(pairs)),
                                       u = Dict(m => s * u_bar[i] for (i, m) in enumerate(umids)))
        return NoTangent(), tangent, Dict(mid => s .* g for (mid, g) in w_bar)
    end
    return f[], free_energy_pullback
end

# Contour steps of one chain on device buffers the caller owns (CuArray pointers), with no
# device allocation by the engine (pf_propagate_noalloc); `stream` is a CUDA stream handle
# (C_NULL: default stream).  Returns once the work is queued; call
# propagate_noalloc_status(stream) after it to learn whether a pencil pass timed out.
function propagate_noalloc!(hist::Ptr, lw::Ptr, ld::Ptr, dims::NTuple{3,Int}, nsteps::Integer;
                            precision::Integer = 0, stream::Ptr{Cvoid} = C_NULL)
    st = ccall((:pf_propagate_noalloc, lib), Cint,
               (Cint, Cint, Cint, Cint, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cvoid}),
               dims[1], dims[2], dims[3], precision, hist, lw, ld, nsteps, stream)
    check(C_NULL, st)
end

propagate_noalloc_status(stream::Ptr{Cvoid} = C_NULL) =
    check(C_NULL, ccall((:pf_propagate_noalloc_status, lib), Cint, (Ptr{Cvoid},), stream))

end # module
