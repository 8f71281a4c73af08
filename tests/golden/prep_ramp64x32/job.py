gas_model = IdealGas(R=287.0)
gas_state = GasState()
gas_state.T = 300.0
gas_state.p = 101325.0
gas_model.update_thermo_from_pT(gas_state)
flow_state = FlowState(gas=gas_state, vx=2.0 * gas_model.speed_of_sound(gas_state), vy=0.0)

config.convective_flux = ConvectiveFlux(flux_calculator=Hanel(), reconstruction_order=2)
config.gas_model = gas_model
config.solver = RungeKutta(cfl=0.5, max_step=500, max_time=1.0, plot_frequency=-1.0, print_frequency=100)
config.grid = Block(
    file_name="ramp.su2",
    initial_condition=flow_state,
    boundaries={
        "inflow": supersonic_inflow(flow_state),
        "outflow": supersonic_outflow(),
        "wall": slip_wall(),
        "top": slip_wall(),
    },
)
